// Device-wide exclusive prefix sum of int32 counts into int64 offsets.
//
// Three passes: each 1024-thread block scans 4096 counts and writes its block
// total, the block totals are scanned the same way (recursively), and the
// block offsets are added back.  Used by the per-cell sort and the bin layout;
// neither runs on the per-step path.
#pragma once

#include "common.cuh"

namespace sg {
namespace {

constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

template <class In>
__global__ void k_scan_block( const In *__restrict__ in, int64_t n, int64_t *__restrict__ out,
                              int64_t *__restrict__ block_sums )
{
    __shared__ int64_t warp_tot[SCAN_THREADS / 32];
    const int64_t base = ( int64_t )blockIdx.x * SCAN_TILE + ( int64_t )threadIdx.x * SCAN_ITEMS;
    int64_t v[SCAN_ITEMS];
    int64_t local = 0;
#pragma unroll
    for( int i = 0; i < SCAN_ITEMS; i++ ) {
        v[i] = base + i < n ? ( int64_t )in[base + i] : 0;
        local += v[i];
    }
    // inclusive warp scan of the per-thread totals
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t x = local;
#pragma unroll
    for( int o = 1; o < 32; o <<= 1 ) {
        int64_t y = __shfl_up_sync( 0xffffffffu, x, o );
        if( lane >= o ) x += y;
    }
    if( lane == 31 ) warp_tot[warp] = x;
    __syncthreads();
    if( warp == 0 ) {
        int64_t w = lane < SCAN_THREADS / 32 ? warp_tot[lane] : 0;
#pragma unroll
        for( int o = 1; o < 32; o <<= 1 ) {
            int64_t y = __shfl_up_sync( 0xffffffffu, w, o );
            if( lane >= o ) w += y;
        }
        if( lane < SCAN_THREADS / 32 ) warp_tot[lane] = w;
    }
    __syncthreads();
    int64_t run = x - local + ( warp > 0 ? warp_tot[warp - 1] : 0 );
#pragma unroll
    for( int i = 0; i < SCAN_ITEMS; i++ ) {
        if( base + i < n ) out[base + i] = run;
        run += v[i];
    }
    if( threadIdx.x == SCAN_THREADS - 1 && block_sums ) block_sums[blockIdx.x] = run;
}

__global__ void k_scan_add( int64_t *__restrict__ out, int64_t n, const int64_t *__restrict__ block_off )
{
    const int64_t i = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x;
    if( i < n ) out[i] += block_off[i / SCAN_TILE];
}

// Scratch (in int64 elements) needed by exclusive_scan for n inputs.
inline int64_t scan_scratch_elems( int64_t n )
{
    int64_t total = 0;
    while( n > SCAN_TILE ) {
        n = ( n + SCAN_TILE - 1 ) / SCAN_TILE;
        total += 2 * n + 2;
    }
    return total + 2;
}

// out[i] = sum_{j<i} in[j]; scratch must hold scan_scratch_elems(n) int64.
template <class In>
inline int exclusive_scan( const In *in, int64_t n, int64_t *out, int64_t *scratch, cudaStream_t s )
{
    if( n <= 0 ) return SG_OK;
    const int64_t nblocks = ( n + SCAN_TILE - 1 ) / SCAN_TILE;
    if( nblocks == 1 ) {
        k_scan_block<In><<<1, SCAN_THREADS, 0, s>>>( in, n, out, nullptr );
        SG_LAUNCH_CHECK( "k_scan_block" );
        return SG_OK;
    }
    int64_t *sums = scratch;
    int64_t *sums_off = scratch + nblocks + 1;
    k_scan_block<In><<<( unsigned )nblocks, SCAN_THREADS, 0, s>>>( in, n, out, sums );
    SG_LAUNCH_CHECK( "k_scan_block" );
    int st = exclusive_scan<int64_t>( sums, nblocks, sums_off, sums_off + nblocks + 1, s );
    if( st ) return st;
    k_scan_add<<<grid_for( n, 256 ), 256, 0, s>>>( out, n, sums_off );
    SG_LAUNCH_CHECK( "k_scan_add" );
    return SG_OK;
}

} // namespace
} // namespace sg
