// Shared helpers of libsmileigb300: error reporting, launch checks and the
// order-2 shape functions used by every particle kernel.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <string>

#include "smilei_gb300.h"

namespace sg {

// Records the calling thread's last error message; returns `code`.
int set_error( int code, const char *fmt, ... );

inline int cuda_fail( cudaError_t e, const char *what, const char *file, int line )
{
    return set_error( SG_ERR_CUDA, "%s failed at %s:%d: %s", what, file, line, cudaGetErrorString( e ) );
}

#define SG_CUDA_TRY( call )                                                                  \
    do {                                                                                     \
        cudaError_t sg_e_ = ( call );                                                        \
        if( sg_e_ != cudaSuccess ) return ::sg::cuda_fail( sg_e_, #call, __FILE__, __LINE__ ); \
    } while( 0 )

#define SG_LAUNCH_CHECK( what ) SG_CUDA_TRY( cudaGetLastError() )

// Releases device memory in cleanup paths; a failure there is not reported and
// must not stay pending as the thread's last error.
inline void release( void *p )
{
    if( p && cudaFree( p ) != cudaSuccess ) cudaGetLastError();
}
inline void release_async( void *p, cudaStream_t s )
{
    if( p && cudaFreeAsync( p, s ) != cudaSuccess ) cudaGetLastError();
}

#define SG_REQUIRE( cond, ... )                                        \
    do {                                                               \
        if( !( cond ) ) return ::sg::set_error( SG_ERR_ARG, __VA_ARGS__ ); \
    } while( 0 )

inline cudaStream_t as_stream( sg_stream_t s ) { return reinterpret_cast<cudaStream_t>( s ); }

inline unsigned grid_for( int64_t n, int block ) { return ( unsigned )( ( n + block - 1 ) / block ); }

// Quadratic B-spline weights at node offsets -1, 0, +1 for an in-cell offset d
// (the reference's Interpolator3D2Order::coeffs, Interpolator3D2Order.h:109-125).
template <class T>
__device__ __forceinline__ void bspline2( T d, T &c0, T &c1, T &c2 )
{
    const T d2 = d * d;
    c0 = T( 0.5 ) * ( d2 - d + T( 0.25 ) );
    c1 = T( 0.75 ) - d2;
    c2 = T( 0.5 ) * ( d2 + d + T( 0.25 ) );
}

__device__ __forceinline__ int round_half_away( double x ) { return ( int )round( x ); }
__device__ __forceinline__ int round_half_away( float x ) { return ( int )roundf( x ); }

// Device error word: the first failing kernel records its code, the host reads it.
struct DeviceStatus {
    int code;
    int detail;
};

} // namespace sg
