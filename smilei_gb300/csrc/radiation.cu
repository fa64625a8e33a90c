// Monte-Carlo radiation reaction and its learned inverse-CDF surrogate.
//
// Tables (FP64, the reference's conventions, src/Radiation/Table.cpp:77-110):
//   integfochi[n]            on log10-spaced chi in [min, max]
//   xi[n_chi, n_ph]          cumulative photon-chi distribution per particle chi
//   axis1_min[n_chi]         log10 of the smallest photon chi of each row
// Kernels:
//   photon-chi inverse CDF   RadiationTables::computeRandomPhotonChiWithInterpolation
//                            (src/Radiation/RadiationTables.cpp:375-512)
//   production yield         computePhotonProductionYield (:225-262)
//   Monte-Carlo pass         RadiationMonteCarlo::operator() (src/Radiation/RadiationMonteCarlo.cpp:62-611),
//                            emitted energy tallied (no macro-photons)
// Learned part: an FP32 MLP 2 -> H -> H -> 1 (tanh) maps (log10 chi, logit10(xi) / 3) to
// log10(photon chi / chi).  It is trained on the GPU by the kernels below
// (forward, backward, batch-reduced weight gradients, Adam) on samples whose
// targets come from the table kernel, validated per (chi, xi) bin against the
// table, and used in the Monte-Carlo pass only where its measured error is
// within tolerance; elsewhere the table answers.
//
// Random numbers: each particle draws from its own counter-based stream,
// fmix32(seed ^ fmix32(id) ^ fmix32(step + 0x9e3779b9)) (MurmurHash3's 32-bit
// finaliser) advanced by xorshift32 (Marsaglia 2003, as the reference's
// src/Tools/Random.h:9-20) and mapped to (0, 1) by x / 2^32 (Random::uniform,
// Random.h:74-75,129, the draw of RadiationMonteCarlo::operator()).

#include "common.cuh"
#include "resident_rad.cuh"

#include <cuda_fp16.h>

#include <cmath>
#include <vector>

namespace sg {
namespace {

struct RadTab {
    const double *integ;
    int n_integ;
    double integ_l0, integ_d, integ_id;
    const double *xi;
    int n_chi, n_ph;
    double xi_l0, xi_d, xi_id, inv_nph_m1;
    const double *axis1_min;
    double factor_dNph_dt, factor_classical, min_cont, min_disc, inv_es;
    const float *integf, *xif, *axis1_minf; // FP32 copies for the FP32-math Monte Carlo
};

__host__ __device__ inline uint32_t fmix32( uint32_t h )
{
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}

__device__ __forceinline__ uint32_t rng_init( uint32_t seed, uint32_t id, uint32_t step )
{
    const uint32_t s = fmix32( seed ^ fmix32( id ) ^ fmix32( step + 0x9e3779b9u ) );
    return s ? s : 0xffffffffu;
}

__device__ __forceinline__ double rng_uniform( uint32_t &s )
{
    s ^= s << 13;
    s ^= s >> 17;
    s ^= s << 5;
    return ( double )s * ( 1.0 / 4294967296.0 );
}

// Radiation::computeParticleChi (src/Radiation/Radiation.h:71-80) in FP64; k = |q/m^2| / E_Schwinger.
__device__ __forceinline__ double particle_chi64( double k, double px, double py, double pz, double Ex, double Ey,
                                                  double Ez, double Bx, double By, double Bz )
{
    const double g = sqrt( 1.0 + px * px + py * py + pz * pz );
    const double a = Ex * px + Ey * py + Ez * pz;
    const double b = g * Ex - By * pz + Bz * py;
    const double c = g * Ey - Bz * px + Bx * pz;
    const double d = g * Ez - Bx * py + By * px;
    return k * sqrt( fabs( a * a - b * b - c * c - d * d ) );
}

// userFunctions::searchValuesInMonotonicArray (src/Tools/userFunctions.h:248-272)
__device__ __forceinline__ int search_monotonic( const double *__restrict__ a, double v, int n )
{
    int imin = 0, imax = n - 1;
    if( v == a[0] ) return 0;
    if( v == a[n - 1] ) return n - 2;
    while( imax - imin > 1 ) {
        const int imid = ( imin + imax ) / 2;
        if( v >= a[imid] ) imin = imid;
        else imax = imid;
    }
    return imin;
}

__device__ double tab_yield( const RadTab &t, double chi, double gamma )
{
    const double lc = log10( chi );
    const int i = ( int )floor( ( lc - t.integ_l0 ) * t.integ_id );
    double v;
    if( i < 0 ) v = t.integ[0];
    else if( i >= t.n_integ - 1 ) v = t.integ[t.n_integ - 2];
    else {
        const double lm = i * t.integ_d + t.integ_l0, lp = lm + t.integ_d;
        v = ( t.integ[i + 1] * fabs( lc - lm ) + t.integ[i] * fabs( lp - lc ) ) * t.integ_id;
    }
    return t.factor_dNph_dt * v * chi / gamma;
}

__device__ double tab_photon_chi( const RadTab &t, double chi, double xi )
{
    const int n1 = t.n_ph;
    const double lc = log10( chi );
    int ic = ( int )floor( ( lc - t.xi_l0 ) * t.xi_id );
    if( ic < 0 ) ic = 0;
    else if( ic > t.n_chi - 2 ) ic = t.n_chi - 2;
    int i1, i2;
    if( xi <= t.xi[ic * n1] ) {
        i1 = 0;
        i2 = 0;
        xi = t.xi[ic * n1];
    } else {
        i1 = search_monotonic( &t.xi[ic * n1], xi, n1 );
        i2 = search_monotonic( &t.xi[( ic + 1 ) * n1], xi, n1 );
    }
    const double dchi = ( lc - ( ic * t.xi_d + t.xi_l0 ) ) * t.xi_id;
    const double d1 = ( ic * t.xi_d + t.xi_l0 - t.axis1_min[ic] ) * t.inv_nph_m1;
    const double d2 = ( ( ic + 1 ) * t.xi_d + t.xi_l0 - t.axis1_min[ic + 1] ) * t.inv_nph_m1;
    const int x1 = ic * n1 + i1, x2 = ( ic + 1 ) * n1 + i2;
    double p1, p2;
    if( t.xi[x1] < 1.0 && t.xi[x1 + 1] - t.xi[x1] > 1e-15 ) {
        const double lm = i1 * d1 + t.axis1_min[ic], lp = lm + d1;
        const double d = ( xi - t.xi[x1] ) / ( t.xi[x1 + 1] - t.xi[x1] );
        p1 = lm * ( 1.0 - d ) + lp * d;
    } else {
        p1 = i1 * d1 + t.axis1_min[ic];
    }
    if( t.xi[x2] < 1.0 && t.xi[x2 + 1] - t.xi[x2] > 1e-15 ) {
        const double lm = i2 * d2 + t.axis1_min[ic + 1], lp = lm + d2;
        const double d = ( xi - t.xi[x2] ) / ( t.xi[x2 + 1] - t.xi[x2] );
        p2 = lm * ( 1.0 - d ) + lp * d;
    } else {
        p2 = i2 * d2 + t.axis1_min[ic + 1];
    }
    return pow( 10.0, p1 * ( 1 - dchi ) + p2 * dchi );
}

// ---- the MLP ----------------------------------------------------------------
// The two lookups in FP32 arithmetic (same interpolation rules as above): the
// table itself is a piecewise-linear fit in log space, far coarser than FP32.
__device__ float tab_yield32( const RadTab &t, float chi, float gamma )
{
    const float lc = log10f( chi );
    const float l0 = ( float )t.integ_l0, d = ( float )t.integ_d, id = ( float )t.integ_id;
    const int i = ( int )floorf( ( lc - l0 ) * id );
    float v;
    if( i < 0 ) v = t.integf[0];
    else if( i >= t.n_integ - 1 ) v = t.integf[t.n_integ - 2];
    else {
        const float lm = i * d + l0, lp = lm + d;
        v = ( t.integf[i + 1] * fabsf( lc - lm ) + t.integf[i] * fabsf( lp - lc ) ) * id;
    }
    return ( float )t.factor_dNph_dt * v * chi / gamma;
}

__device__ __forceinline__ int search_monotonic32( const float *__restrict__ a, float v, int n )
{
    int imin = 0, imax = n - 1;
    if( v == a[0] ) return 0;
    if( v == a[n - 1] ) return n - 2;
    while( imax - imin > 1 ) {
        const int imid = ( imin + imax ) / 2;
        if( v >= a[imid] ) imin = imid;
        else imax = imid;
    }
    return imin;
}

__device__ float tab_photon_chi32( const RadTab &t, float chi, float xi )
{
    const int n1 = t.n_ph;
    const float lc = log10f( chi );
    const float l0 = ( float )t.xi_l0, d0 = ( float )t.xi_d, id0 = ( float )t.xi_id, inm1 = ( float )t.inv_nph_m1;
    int ic = ( int )floorf( ( lc - l0 ) * id0 );
    if( ic < 0 ) ic = 0;
    else if( ic > t.n_chi - 2 ) ic = t.n_chi - 2;
    const float *X = t.xif;
    int i1, i2;
    if( xi <= X[ic * n1] ) {
        i1 = 0;
        i2 = 0;
        xi = X[ic * n1];
    } else {
        i1 = search_monotonic32( &X[ic * n1], xi, n1 );
        i2 = search_monotonic32( &X[( ic + 1 ) * n1], xi, n1 );
    }
    const float dchi = ( lc - ( ic * d0 + l0 ) ) * id0;
    const float d1 = ( ic * d0 + l0 - t.axis1_minf[ic] ) * inm1;
    const float d2 = ( ( ic + 1 ) * d0 + l0 - t.axis1_minf[ic + 1] ) * inm1;
    const int x1 = ic * n1 + i1, x2 = ( ic + 1 ) * n1 + i2;
    float p1, p2;
    if( X[x1] < 1.0f && X[x1 + 1] - X[x1] > 1e-15f ) {
        const float lm = i1 * d1 + t.axis1_minf[ic], lp = lm + d1;
        const float d = ( xi - X[x1] ) / ( X[x1 + 1] - X[x1] );
        p1 = lm * ( 1.0f - d ) + lp * d;
    } else {
        p1 = i1 * d1 + t.axis1_minf[ic];
    }
    if( X[x2] < 1.0f && X[x2 + 1] - X[x2] > 1e-15f ) {
        const float lm = i2 * d2 + t.axis1_minf[ic + 1], lp = lm + d2;
        const float d = ( xi - X[x2] ) / ( X[x2 + 1] - X[x2] );
        p2 = lm * ( 1.0f - d ) + lp * d;
    } else {
        p2 = i2 * d2 + t.axis1_minf[ic + 1];
    }
    return exp10f( p1 * ( 1.0f - dchi ) + p2 * dchi );
}

constexpr int MLP_MAX_H = 128;

struct MlpView {
    int H;
    const float *W1, *b1, *W2, *b2, *W3, *b3; // W1[H][2] W2[H][H] W3[H]
    float lmin, lspan;                         // input normalisation of log10 chi
    float out_scale;                           // network output * out_scale = log10(photon chi / chi)
    const int *mask;                           // fallback mask [nbc][nbx] (1 = use the table)
    int nbc, nbx;
};

__host__ __device__ inline int mlp_nparams( int H ) { return H * H + 5 * H + 1; }

// Activation of the inference paths: the hardware tanh approximation (relative error
// below 2^-10, far under the network's own error against the table).  Training uses
// tanhf, whose derivative 1 - h^2 the back-propagation relies on.
__device__ __forceinline__ float tanh_fast( float x )
{
    float y;
    asm( "tanh.approx.f32 %0, %1;" : "=f"( y ) : "f"( x ) );
    return y;
}

template <bool FAST>
__device__ __forceinline__ float act( float x )
{
    if constexpr( FAST ) return tanh_fast( x );
    else return tanhf( x );
}

// Forward pass of one sample; optional activations out.  FAST: inference activation.
template <bool FAST = false>
__device__ __forceinline__ float mlp_forward( const MlpView &m, float u0, float u1, float *h1, float *h2 )
{
    const int H = m.H;
    for( int i = 0; i < H; i++ ) h1[i] = act<FAST>( m.W1[2 * i] * u0 + m.W1[2 * i + 1] * u1 + m.b1[i] );
    float y = m.b3[0];
    for( int i = 0; i < H; i++ ) {
        float a = m.b2[i];
        const float *w = m.W2 + i * H;
        for( int j = 0; j < H; j++ ) a = fmaf( w[j], h1[j], a );
        h2[i] = act<FAST>( a );
        y = fmaf( m.W3[i], h2[i], y );
    }
    return y;
}

// The network's xi input: log10(xi / (1 - xi)) / 3, xi clamped to [1e-7, 1 - 2^-23].  The
// inverse CDF is steep in xi at both ends (about 3 log10 xi near 0, a log of 1 - xi near
// 1) and nearly linear in this coordinate.
__device__ __forceinline__ float mlp_xi_input( float xi )
{
    xi = fminf( fmaxf( xi, 1e-7f ), 1.0f - 1.1920929e-7f );
    return ( log10f( xi ) - log10f( 1.0f - xi ) ) * ( 1.0f / 3.0f );
}

__device__ __forceinline__ void mlp_inputs( const MlpView &m, double chi, double xi, float &u0, float &u1 )
{
    u0 = 2.0f * ( ( float )log10( chi ) - m.lmin ) / m.lspan - 1.0f;
    u1 = mlp_xi_input( ( float )xi );
}

__device__ double mlp_photon_chi( const MlpView &m, double chi, double xi )
{
    float h1[MLP_MAX_H], h2[MLP_MAX_H];
    float u0, u1;
    mlp_inputs( m, chi, xi, u0, u1 );
    const float y = mlp_forward<true>( m, u0, u1, h1, h2 );
    return chi * ( double )exp10f( y * m.out_scale );
}

__device__ __forceinline__ bool mlp_masked( const MlpView &m, double chi, double xi )
{
    float u0 = ( ( float )log10( chi ) - m.lmin ) / m.lspan;
    int bc = ( int )floorf( u0 * m.nbc ), bx = ( int )floor( xi * m.nbx );
    if( bc < 0 || bc >= m.nbc ) return true; // outside the trained range
    bx = bx < 0 ? 0 : ( bx >= m.nbx ? m.nbx - 1 : bx );
    return m.mask[bc * m.nbx + bx] != 0;
}

// ---- kernels ------------------------------------------------------------------
__global__ void k_photon_chi( RadTab t, int64_t n, const double *__restrict__ chi, const double *__restrict__ xi,
                              double *__restrict__ out )
{
    const int64_t i = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x;
    if( i < n ) out[i] = tab_photon_chi( t, chi[i], xi[i] );
}

__global__ void k_yield( RadTab t, int64_t n, const double *__restrict__ chi, const double *__restrict__ g,
                         double *__restrict__ out )
{
    const int64_t i = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x;
    if( i < n ) out[i] = tab_yield( t, chi[i], g[i] );
}

__global__ void k_mlp_photon_chi( MlpView m, int64_t n, const double *__restrict__ chi, const double *__restrict__ xi,
                                  double *__restrict__ out )
{
    const int64_t i = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x;
    if( i < n ) out[i] = mlp_photon_chi( m, chi[i], xi[i] );
}

// Batched inference for a compile-time width: the parameters are staged once per
// block in shared memory (every thread reads the same weight: broadcasts), the
// hidden activations stay in registers, and the output power is taken in FP32
// (FP64 is slow on this GPU; the network's own error is far above FP32 rounding).
template <int H>
__global__ void __launch_bounds__( 256 ) k_mlp_photon_chi_fast( MlpView m, int64_t n, const double *__restrict__ chi,
                                                                const double *__restrict__ xi, double *__restrict__ out )
{
    __shared__ float sW1[2 * H], sb1[H], sb2[H], sW3[H], sb3;
    __shared__ float4 sW2v[H * H / 4]; // row r, columns 4c..4c+3 at r * H / 4 + c
    float *sW2 = reinterpret_cast<float *>( sW2v );
    for( int k = threadIdx.x; k < H * H; k += blockDim.x ) sW2[k] = m.W2[k];
    for( int k = threadIdx.x; k < H; k += blockDim.x ) {
        sW1[2 * k] = m.W1[2 * k];
        sW1[2 * k + 1] = m.W1[2 * k + 1];
        sb1[k] = m.b1[k];
        sb2[k] = m.b2[k];
        sW3[k] = m.W3[k];
    }
    if( threadIdx.x == 0 ) sb3 = m.b3[0];
    __syncthreads();
    for( int64_t i = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x; i < n; i += ( int64_t )gridDim.x * blockDim.x ) {
        const float c = ( float )chi[i];
        const float u0 = 2.0f * ( log10f( c ) - m.lmin ) / m.lspan - 1.0f;
        const float u1 = mlp_xi_input( ( float )xi[i] );
        float h1[H];
#pragma unroll
        for( int k = 0; k < H; k++ ) h1[k] = tanh_fast( fmaf( sW1[2 * k], u0, fmaf( sW1[2 * k + 1], u1, sb1[k] ) ) );
        float y = sb3;
#pragma unroll( H >= 64 ? 1 : 2 )
        for( int r = 0; r < H; r++ ) {
            float a = sb2[r];
#pragma unroll
            for( int c = 0; c < H / 4; c++ ) {
                const float4 wv = sW2v[r * ( H / 4 ) + c];
                a = fmaf( wv.x, h1[4 * c], a );
                a = fmaf( wv.y, h1[4 * c + 1], a );
                a = fmaf( wv.z, h1[4 * c + 2], a );
                a = fmaf( wv.w, h1[4 * c + 3], a );
            }
            y = fmaf( sW3[r], tanh_fast( a ), y );
        }
        out[i] = chi[i] * ( double )exp10f( y * m.out_scale );
    }
}

// Batched inference of the 64-wide network on the tensor cores (mma.sync
// m16n8k16, FP16 operands, FP32 accumulation): a warp takes 32 samples at a time
// (two 16-row tiles).  Layer 1 (2 -> 64) and both activations run on the FP32 cores,
// each lane computing exactly the hidden values its operand fragments hold; layer 2
// (64 x 64, 96 % of the network's arithmetic) is 64 mma instructions per 32 samples;
// layer 3 is a sum over the accumulator fragments and two shuffles.  FP16 rounding of
// the hidden values and of W2 (relative 2^-11) is far below the network's own error
// against the table; the test bounds the difference to the FP32 network.
constexpr int TC_H = 64;
constexpr int TC_W2_STRIDE = TC_H + 8; // halves per row of W2 in shared memory: no bank conflicts

__device__ __forceinline__ uint32_t pack_half2( float lo, float hi )
{
    const __half2 h = __floats2half2_rn( lo, hi );
    return *reinterpret_cast<const uint32_t *>( &h );
}

// The 64-wide network on one warp for up to 16 MT rows (MT 16-row tiles together; mtiles
// < MT uses only the first mtiles): ru0/ru1 hold the inputs of rows 16 mt + gid + 8 hf, the rows this
// lane's fragments hold (gid = lane / 4, tig = lane % 4).  Returns in y[mt][hf] the
// output before b3 of those rows, complete in all four lanes of the group.  W2h: FP16
// W2 (row = output unit) with rows TC_W2_STRIDE halves apart.
template <int MT>
__device__ __forceinline__ void tc_network( const __half *__restrict__ W2h, const float *__restrict__ W1,
                                            const float *__restrict__ b1, const float *__restrict__ b2,
                                            const float *__restrict__ W3, const float ( &ru0 )[MT][2],
                                            const float ( &ru1 )[MT][2], int mtiles, float ( &y )[MT][2] )
{
    const int lane = threadIdx.x & 31, gid = lane >> 2, tig = lane & 3;
    float acc[MT][8][4];
#pragma unroll
    for( int mt = 0; mt < MT; mt++ )
#pragma unroll
        for( int nt = 0; nt < 8; nt++ )
#pragma unroll
            for( int e = 0; e < 4; e++ ) acc[mt][nt][e] = 0.0f;
#pragma unroll
    for( int ks = 0; ks < 4; ks++ ) {
        // layer 1 for the columns k = 16 ks + 2 tig + {0, 1} (+ 8) of this lane's rows
        uint32_t a[MT][4];
#pragma unroll
        for( int mt = 0; mt < MT; mt++ )
#pragma unroll
            for( int r = 0; r < 4; r++ ) { // r: (hf, kh) = (r & 1, r >> 1), the PTX order a0..a3
                const int hf = r & 1, k0 = 16 * ks + 2 * tig + 8 * ( r >> 1 );
                const float v0 = tanh_fast( fmaf( W1[2 * k0], ru0[mt][hf], fmaf( W1[2 * k0 + 1], ru1[mt][hf], b1[k0] ) ) );
                const float v1 = tanh_fast( fmaf( W1[2 * k0 + 2], ru0[mt][hf], fmaf( W1[2 * k0 + 3], ru1[mt][hf], b1[k0 + 1] ) ) );
                a[mt][r] = pack_half2( v0, v1 );
            }
#pragma unroll
        for( int nt = 0; nt < 8; nt++ ) {
            const __half *wrow = W2h + ( 8 * nt + gid ) * TC_W2_STRIDE + 16 * ks + 2 * tig;
            const uint32_t b0 = *reinterpret_cast<const uint32_t *>( wrow );
            const uint32_t bb = *reinterpret_cast<const uint32_t *>( wrow + 8 );
#pragma unroll
            for( int mt = 0; mt < MT; mt++ )
                if( mt < mtiles )
                    asm volatile( "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
                                  "{%8,%9}, {%0,%1,%2,%3};\n"
                                  : "+f"( acc[mt][nt][0] ), "+f"( acc[mt][nt][1] ), "+f"( acc[mt][nt][2] ),
                                    "+f"( acc[mt][nt][3] )
                                  : "r"( a[mt][0] ), "r"( a[mt][1] ), "r"( a[mt][2] ), "r"( a[mt][3] ), "r"( b0 ),
                                    "r"( bb ) );
        }
    }
    // layer 2 activation and layer 3: rows gid (+ 8) of each tile, columns 8 nt + 2 tig + {0, 1}
#pragma unroll
    for( int mt = 0; mt < MT; mt++ ) {
        y[mt][0] = y[mt][1] = 0.0f;
#pragma unroll
        for( int nt = 0; nt < 8; nt++ )
#pragma unroll
            for( int e = 0; e < 4; e++ ) {
                const int col = 8 * nt + 2 * tig + ( e & 1 );
                y[mt][e >> 1] = fmaf( W3[col], tanh_fast( acc[mt][nt][e] + b2[col] ), y[mt][e >> 1] );
            }
    }
#pragma unroll
    for( int mt = 0; mt < MT; mt++ )
#pragma unroll
        for( int hf = 0; hf < 2; hf++ ) {
            y[mt][hf] += __shfl_xor_sync( 0xffffffffu, y[mt][hf], 1 );
            y[mt][hf] += __shfl_xor_sync( 0xffffffffu, y[mt][hf], 2 );
        }
}

// Row k's output (k < 32) from the group that holds it: lanes 4 (k % 8) .. + 3.
__device__ __forceinline__ float tc_row( const float ( &y )[2][2], int k )
{
    const int src = 4 * ( k & 7 );
    const float y00 = __shfl_sync( 0xffffffffu, y[0][0], src ), y01 = __shfl_sync( 0xffffffffu, y[0][1], src );
    const float y10 = __shfl_sync( 0xffffffffu, y[1][0], src ), y11 = __shfl_sync( 0xffffffffu, y[1][1], src );
    return ( k >> 4 ) ? ( ( k >> 3 ) & 1 ? y11 : y10 ) : ( ( k >> 3 ) & 1 ? y01 : y00 );
}

__global__ void __launch_bounds__( 128 ) k_mlp_photon_chi_tc( MlpView m, int64_t n, const double *__restrict__ chi,
                                                              const double *__restrict__ xi, double *__restrict__ out )
{
    __shared__ __align__( 16 ) __half sW2[TC_H * TC_W2_STRIDE];
    __shared__ float sW1[2 * TC_H], sb1[TC_H], sb2[TC_H], sW3[TC_H];
    for( int k = threadIdx.x; k < TC_H * TC_H; k += blockDim.x )
        sW2[( k / TC_H ) * TC_W2_STRIDE + ( k % TC_H )] = __float2half_rn( m.W2[k] );
    for( int k = threadIdx.x; k < TC_H; k += blockDim.x ) {
        sW1[2 * k] = m.W1[2 * k];
        sW1[2 * k + 1] = m.W1[2 * k + 1];
        sb1[k] = m.b1[k];
        sb2[k] = m.b2[k];
        sW3[k] = m.W3[k];
    }
    __syncthreads();
    const float b3 = m.b3[0];
    const int lane = threadIdx.x & 31, gid = lane >> 2, tig = lane & 3;
    const int64_t warps = ( int64_t )gridDim.x * ( blockDim.x >> 5 );
    for( int64_t base = ( ( int64_t )blockIdx.x * ( blockDim.x >> 5 ) + ( threadIdx.x >> 5 ) ) * 32; base < n;
         base += warps * 32 ) {
        // this lane's own sample (row `lane` of the 32)
        const int64_t i = base + lane;
        float c = 1.0f, u0 = 0.0f, u1 = 0.0f;
        if( i < n ) {
            c = ( float )chi[i];
            u0 = 2.0f * ( log10f( c ) - m.lmin ) / m.lspan - 1.0f;
            u1 = mlp_xi_input( ( float )xi[i] );
        }
        // inputs of the four rows this lane's fragments hold: 16 mt + gid + 8 hf
        float ru0[2][2], ru1[2][2];
#pragma unroll
        for( int mt = 0; mt < 2; mt++ )
#pragma unroll
            for( int hf = 0; hf < 2; hf++ ) {
                ru0[mt][hf] = __shfl_sync( 0xffffffffu, u0, 16 * mt + gid + 8 * hf );
                ru1[mt][hf] = __shfl_sync( 0xffffffffu, u1, 16 * mt + gid + 8 * hf );
            }
        float y[2][2];
        tc_network<2>( sW2, sW1, sb1, sb2, sW3, ru0, ru1, 2, y );
        const float yl = tc_row( y, lane );
        if( i < n ) out[i] = chi[i] * ( double )exp10f( ( yl + b3 ) * m.out_scale );
    }
}

// Macro-photon output (RadiationMonteCarlo.cpp:425-545): an emission with
// photon_gamma >= threshold, while the particle has made fewer than max_emissions
// photons in this pass, appends `sampling` photons (slots from one atomicAdd on
// count) at the particle's position, momentum photon_gamma p / |p| with p after
// the recoil, weight w / sampling, chi = photon chi, tau = -1; its energy is then
// not tallied as radiated.  Slots at or past cap are not written.  count == null:
// no photons.
struct PhotonOut {
    const double *pos;
    int ndim, sampling, max_emissions;
    double threshold;
    int64_t cap;
    unsigned long long *count;
    double *ph_pos, *ph_mom, *ph_w, *ph_chi, *ph_tau; // ph_pos[d * cap + k], ph_mom[c * cap + k]
    double dx[2]; // resident photons: cell lengths, a photon starting at (node + offset) dx
};

// RadiationMonteCarlo::operator() per particle (see the file header).
// The network's weights in shared memory, for kernels that evaluate it per thread.
template <int H>
struct MlpShared {
    float W1[2 * H], b1[H], b2[H], W3[H], b3;
    float4 W2v[H * H / 4]; // row r, columns 4c..4c+3 at r * H / 4 + c
};
// The 64-wide network is evaluated on the tensor cores (tc_network): W2 in FP16.
template <>
struct MlpShared<TC_H> {
    float W1[2 * TC_H], b1[TC_H], b2[TC_H], W3[TC_H], b3;
    __align__( 16 ) __half W2h[TC_H * TC_W2_STRIDE];
};

// TRANSPOSED: W2 stored column-major (W2T[i * H + r] = W2[r][i]) for the
// warp-cooperative evaluation, where lane r reads row r of consecutive columns.
template <int H, bool TRANSPOSED = false>
__device__ __forceinline__ void mlp_stage( const MlpView &m, MlpShared<H> &w )
{
    if constexpr( H == TC_H ) {
        for( int k = threadIdx.x; k < H * H; k += blockDim.x )
            w.W2h[( k / H ) * TC_W2_STRIDE + ( k % H )] = __float2half_rn( m.W2[k] );
    } else {
        float *W2 = reinterpret_cast<float *>( w.W2v );
        for( int k = threadIdx.x; k < H * H; k += blockDim.x ) {
            if constexpr( TRANSPOSED ) W2[( k % H ) * H + k / H] = m.W2[k];
            else W2[k] = m.W2[k];
        }
    }
    for( int k = threadIdx.x; k < H; k += blockDim.x ) {
        w.W1[2 * k] = m.W1[2 * k];
        w.W1[2 * k + 1] = m.W1[2 * k + 1];
        w.b1[k] = m.b1[k];
        w.b2[k] = m.b2[k];
        w.W3[k] = m.W3[k];
    }
    if( threadIdx.x == 0 ) w.b3 = m.b3[0];
}

// photon chi = chi 10^(out_scale * network(log10 chi, xi)), hidden layer in registers
template <int H>
__device__ __forceinline__ double mlp_photon_chi_smem( const MlpView &m, const MlpShared<H> &w, double chi, double xi )
{
    // one sample per thread: the 64-wide network reads its FP32 weights from global memory
    if constexpr( H == TC_H ) {
        return mlp_photon_chi( m, chi, xi );
    } else {
        const float u0 = 2.0f * ( log10f( ( float )chi ) - m.lmin ) / m.lspan - 1.0f;
        const float u1 = mlp_xi_input( ( float )xi );
        float h1[H];
#pragma unroll
        for( int k = 0; k < H; k++ ) h1[k] = tanh_fast( fmaf( w.W1[2 * k], u0, fmaf( w.W1[2 * k + 1], u1, w.b1[k] ) ) );
        float y = w.b3;
#pragma unroll( H >= 64 ? 1 : 2 )
        for( int r = 0; r < H; r++ ) {
            float a = w.b2[r];
#pragma unroll
            for( int c = 0; c < H / 4; c++ ) {
                const float4 wv = w.W2v[r * ( H / 4 ) + c];
                a = fmaf( wv.x, h1[4 * c], a );
                a = fmaf( wv.y, h1[4 * c + 1], a );
                a = fmaf( wv.z, h1[4 * c + 2], a );
                a = fmaf( wv.w, h1[4 * c + 3], a );
            }
            y = fmaf( w.W3[r], tanh_fast( a ), y );
        }
        return chi * ( double )exp10f( y * m.out_scale );
    }
}

// The network evaluated by a whole warp for one (chi, xi) (every lane passes the
// same values; W2 staged transposed): lane l owns hidden units l and l + 32, the
// first layer's outputs travel by shuffles, the last layer is a warp sum.  About
// H shuffles and 2H FMAs per lane instead of H^2 FMAs in one thread.
template <int H>
__device__ __forceinline__ float mlp_coop( const MlpView &m, const MlpShared<H> &w, float chi, float xi, int lane )
{
    constexpr int K = H >= 32 ? H / 32 : 1;
    const float u0 = 2.0f * ( log10f( chi ) - m.lmin ) / m.lspan - 1.0f;
    const float u1 = mlp_xi_input( xi );
    const float *W2T = reinterpret_cast<const float *>( w.W2v );
    float h[K], acc[K];
#pragma unroll
    for( int k = 0; k < K; k++ ) {
        const int j = lane + 32 * k;
        h[k] = j < H ? tanh_fast( fmaf( w.W1[2 * j], u0, fmaf( w.W1[2 * j + 1], u1, w.b1[j] ) ) ) : 0.0f;
        acc[k] = j < H ? w.b2[j] : 0.0f;
    }
#pragma unroll 8
    for( int i = 0; i < H; i++ ) {
        const float hv = __shfl_sync( 0xffffffffu, h[i >> 5], i & 31 );
#pragma unroll
        for( int k = 0; k < K; k++ ) {
            const int r = lane + 32 * k;
            if( r < H ) acc[k] = fmaf( W2T[i * H + r], hv, acc[k] );
        }
    }
    float y = 0.0f;
#pragma unroll
    for( int k = 0; k < K; k++ ) {
        const int r = lane + 32 * k;
        if( r < H ) y = fmaf( w.W3[r], tanh_fast( acc[k] ), y );
    }
#pragma unroll
    for( int o = 16; o > 0; o >>= 1 ) y += __shfl_xor_sync( 0xffffffffu, y, o );
    return y + w.b3;
}

// One particle's Monte-Carlo steps over dt in FP32 arithmetic for gamma, chi, the
// rates, times and the optical depth (the momenta and the radiated-energy tally stay
// FP64), RadiationMonteCarlo::operator() (RadiationMonteCarlo.cpp:62-611).  Called by
// every lane of a warp (inactive lanes too): the loop is warp-synchronous, so that the
// lanes that emit through the network evaluate it together, one emission after another.
// ph.count == null: no macro-photons (then xp, xn, xo are unused).  Its photons start at
// the particle's position: xp (ph.ndim values) or, with xp null, (xn + xo) ph.dx (node
// and offset; the FP64 position is formed only when a photon is made).
// P: the arithmetic of the momenta and of the recoil (double for FP64 momenta, float
// for the mixed form's FP32 momenta).  PH false: no photon output is compiled in.
template <int H, class P, bool PH = true>
__device__ __forceinline__ void mc_pass_f32( const RadTab &t, const MlpView &m, int use_mlp,
                                             const MlpShared<H == 0 ? 4 : H> &sw, bool active, double dt, double qm2,
                                             const float *E3, const float *B3, P &px, P &py, P &pz,
                                             float &tp, uint32_t &rs, double wgt, double &rad, unsigned long long &nem,
                                             const PhotonOut &ph, const double *xp, const int *xn = nullptr,
                                             const float *xo = nullptr )
{
    const int lane = threadIdx.x & 31;
    const float Ex = E3[0], Ey = E3[1], Ez = E3[2], Bx = B3[0], By = B3[1], Bz = B3[2];
    const float k_chi = ( float )( fabs( qm2 ) * t.inv_es );
    const float dtf = ( float )dt, min_disc = ( float )t.min_disc, min_cont = ( float )t.min_cont;
    // the optical depth counts as spent at or below eps_tau (the FP64 pass uses 1e-100):
    // a residual of the subtraction below it would otherwise never reach zero and
    // stall the particle's emissions
    const float eps_tau = 1e-30f;
    float local_time = 0.0f;
    int it = 0, i_photon = 0;
    while( __any_sync( 0xffffffffu, active ) ) {
        bool emit = false, net = false;
        float g = 0.0f, chi = 0.0f, u32 = 0.0f;
        double pchi = 0.0;
        if( active && !( local_time < dtf && it < 100 ) ) active = false;
        if( active ) {
            const float fx = ( float )px, fy = ( float )py, fz = ( float )pz;
            g = sqrtf( 1.0f + fx * fx + fy * fy + fz * fz );
            if( g < 1.1f ) {
                active = false;
            } else {
                const float a = Ex * fx + Ey * fy + Ez * fz;
                const float b = g * Ex - By * fz + Bz * fy;
                const float c = g * Ey - Bz * fx + Bx * fz;
                const float d = g * Ez - Bx * fy + By * fx;
                chi = k_chi * sqrtf( fabsf( a * a - b * b - c * c - d * d ) );
                if( chi > min_disc && tp <= eps_tau ) {
                    while( tp <= eps_tau ) tp = -logf( fmaxf( 1.0f - ( float )rng_uniform( rs ), 5.9604645e-8f ) );
                }
                if( tp > eps_tau ) {
                    const float rate = tab_yield32( t, chi, g );
                    const float emission_time = fminf( tp / rate, dtf - local_time );
                    tp -= rate * emission_time;
                    if( tp <= eps_tau ) {
                        const double u = rng_uniform( rs );
                        emit = true;
                        if( use_mlp && !mlp_masked( m, chi, u ) ) {
                            if constexpr( H > 0 ) {
                                net = true;
                                u32 = ( float )u;
                            } else {
                                pchi = mlp_photon_chi( m, chi, u );
                            }
                        } else {
                            pchi = ( double )tab_photon_chi32( t, chi, ( float )u );
                        }
                    }
                    it++;
                    local_time += emission_time;
                } else if( chi <= min_disc && tp <= eps_tau && chi > min_cont ) {
                    const float emission_time = dtf - local_time;
                    const float aa = 1.0f + 4.8f * ( 1.0f + chi ) * logf( 1.0f + 1.7f * chi ) + 2.44f * chi * chi;
                    const float e = ( 1.0f / cbrtf( aa * aa ) ) * emission_time * chi * chi * ( float )t.factor_classical;
                    const P tmp = ( P )( e * g / ( g * g - 1.0f ) );
                    const P gd = sqrt( P( 1 ) + px * px + py * py + pz * pz );
                    px -= tmp * px;
                    py -= tmp * py;
                    pz -= tmp * pz;
                    rad += wgt * ( double )( gd - sqrt( P( 1 ) + px * px + py * py + pz * pz ) );
                    local_time = dtf;
                } else {
                    local_time = dtf;
                }
            }
        }
        if constexpr( H == TC_H ) {
            // the emitting lanes' network evaluations as one batch on the tensor cores:
            // row k is the lane with the k-th lowest index among them
            const unsigned req = __ballot_sync( 0xffffffffu, net );
            if( req ) {
                const int nreq = __popc( req );
                float u0 = 0.0f, u1 = 0.0f;
                if( net ) {
                    u0 = 2.0f * ( log10f( chi ) - m.lmin ) / m.lspan - 1.0f;
                    u1 = mlp_xi_input( u32 );
                }
                const int gid = lane >> 2;
                // one 16-row tile at a time (a second only past 16 rows): the accumulators
                // of one tile, not two, stay live in this long loop
                float y00 = 0.0f, y01 = 0.0f, y10 = 0.0f, y11 = 0.0f;
#pragma unroll 1
                for( int mt = 0; mt < 2; mt++ ) {
                    if( mt * 16 >= nreq ) break;
                    float ru0[1][2], ru1[1][2];
#pragma unroll
                    for( int hf = 0; hf < 2; hf++ ) {
                        const int row = 16 * mt + gid + 8 * hf;
                        const int src = row < nreq ? ( int )__fns( req, 0, row + 1 ) : lane;
                        const float a0 = __shfl_sync( 0xffffffffu, u0, src ), a1 = __shfl_sync( 0xffffffffu, u1, src );
                        ru0[0][hf] = row < nreq ? a0 : 0.0f;
                        ru1[0][hf] = row < nreq ? a1 : 0.0f;
                    }
                    float y1[1][2];
                    tc_network<1>( sw.W2h, sw.W1, sw.b1, sw.b2, sw.W3, ru0, ru1, 1, y1 );
                    if( mt == 0 ) {
                        y00 = y1[0][0];
                        y01 = y1[0][1];
                    } else {
                        y10 = y1[0][0];
                        y11 = y1[0][1];
                    }
                }
                const float yv[2][2] = { { y00, y01 }, { y10, y11 } };
                const float y = tc_row( yv, __popc( req & ( ( 1u << lane ) - 1u ) ) );
                if( net ) pchi = ( double )chi * ( double )exp10f( ( y + sw.b3 ) * m.out_scale );
            }
        } else if constexpr( H > 0 ) {
            // the emitting lanes' network evaluations, by the whole warp
            unsigned req = __ballot_sync( 0xffffffffu, net );
            while( req ) {
                const int src = __ffs( req ) - 1;
                req &= req - 1;
                const float cs = __shfl_sync( 0xffffffffu, chi, src ), us = __shfl_sync( 0xffffffffu, u32, src );
                const float y = mlp_coop<H>( m, sw, cs, us, lane );
                if( lane == src ) pchi = ( double )chi * ( double )exp10f( y * m.out_scale );
            }
        }
        if( emit ) {
            const P gd = sqrt( P( 1 ) + px * px + py * py + pz * pz );
            const P pg = ( P )pchi / ( P )chi * ( gd - P( 1 ) );
            const P f = ( P )( ( float )pg / sqrtf( g * g - 1.0f ) );
            px -= px * f;
            py -= py * f;
            pz -= pz * f;
            if( PH && ph.count && ( double )pg >= ph.threshold && i_photon < ph.max_emissions ) {
                const double inv = 1.0 / sqrt( ( double )( px * px + py * py + pz * pz ) );
                const unsigned long long o0 = atomicAdd( ph.count, ( unsigned long long )ph.sampling );
                for( int k = 0; k < ph.sampling; k++ ) {
                    const unsigned long long o = o0 + ( unsigned long long )k;
                    if( o >= ( unsigned long long )ph.cap ) break;
                    for( int dd = 0; dd < ph.ndim; dd++ )
                        ph.ph_pos[dd * ph.cap + o] = xp ? xp[dd] : ( ( double )xn[dd] + ( double )xo[dd] ) * ph.dx[dd];
                    ph.ph_mom[o] = ( double )pg * px * inv;
                    ph.ph_mom[ph.cap + o] = ( double )pg * py * inv;
                    ph.ph_mom[2 * ph.cap + o] = ( double )pg * pz * inv;
                    ph.ph_w[o] = wgt * ( 1.0 / ph.sampling );
                    ph.ph_chi[o] = pchi;
                    ph.ph_tau[o] = -1.0;
                }
                i_photon++;
            } else {
                rad += wgt * ( double )( gd - sqrt( P( 1 ) + px * px + py * py + pz * pz ) );
            }
            nem++;
            tp = -1.0f;
        }
    }
}

// F32: the table lookups, the optical-depth draw and the continuous-loss formula in
// FP32 arithmetic (FP64 is a small fraction of FP32 throughput on this GPU); chi,
// gamma, times and momenta stay FP64.  The random stream is the FP64 pass's.
// H > 0: the network (H hidden units) evaluated from shared memory; H == 0 with
// use_mlp: any width, weights read from global memory.
template <bool F32, int H>
__global__ void k_monte_carlo( RadTab t, MlpView m, int use_mlp, int64_t n, double dt, double qm2,
                               double *__restrict__ mom, const double *__restrict__ w, double *__restrict__ tau,
                               double *__restrict__ chi_out, const double *__restrict__ Ep,
                               const double *__restrict__ Bp, uint32_t seed, uint32_t first_id, uint32_t step,
                               double *__restrict__ radiated, unsigned long long *__restrict__ n_emit, PhotonOut ph )
{
    __shared__ MlpShared<H == 0 ? 4 : H> sw;
    if constexpr( H > 0 ) {
        mlp_stage<H, F32>( m, sw );
        __syncthreads();
    }
    const int64_t p = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x;
    double rad = 0.0;
    unsigned long long nem = 0;
    if( !F32 && p < n ) { // the reference's FP64 arithmetic
        double px = mom[p], py = mom[n + p], pz = mom[2 * n + p];
        const double Ex = Ep[p], Ey = Ep[n + p], Ez = Ep[2 * n + p];
        const double Bx = Bp[p], By = Bp[n + p], Bz = Bp[2 * n + p];
        double tp = tau[p];
        uint32_t rs = rng_init( seed, first_id + ( uint32_t )p, step );
        double local_time = 0.0, emission_time = 0.0;
        int it = 0, i_photon = 0;
        const double eps_tau = 1e-100;
        while( local_time < dt && it < 100 ) {
            const double g = sqrt( 1.0 + px * px + py * py + pz * pz );
            if( g < 1.1 ) break;
            const double a = Ex * px + Ey * py + Ez * pz;
            const double b = g * Ex - By * pz + Bz * py;
            const double c = g * Ey - Bz * px + Bx * pz;
            const double d = g * Ez - Bx * py + By * px;
            const double chi = fabs( qm2 ) * t.inv_es * sqrt( fabs( a * a - b * b - c * c - d * d ) );
            if( chi > t.min_disc && tp <= eps_tau ) {
                while( tp <= eps_tau ) tp = -log( 1.0 - rng_uniform( rs ) );
            }
            if( tp > eps_tau ) {
                const double rate = tab_yield( t, chi, g );
                emission_time = fmin( tp / rate, dt - local_time );
                tp -= rate * emission_time;
                if( tp <= eps_tau ) {
                    const double u = rng_uniform( rs );
                    double pchi;
                    if( use_mlp && !mlp_masked( m, chi, u ) ) {
                        if constexpr( H > 0 ) pchi = mlp_photon_chi_smem<H>( m, sw, chi, u );
                        else pchi = mlp_photon_chi( m, chi, u );
                    } else {
                        pchi = tab_photon_chi( t, chi, u );
                    }
                    const double pg = pchi / chi * ( g - 1.0 );
                    const double f = pg / sqrt( g * g - 1.0 );
                    px -= px * f;
                    py -= py * f;
                    pz -= pz * f;
                    if( ph.count && pg >= ph.threshold && i_photon < ph.max_emissions ) {
                        const double inv = 1.0 / sqrt( px * px + py * py + pz * pz );
                        const unsigned long long o0 = atomicAdd( ph.count, ( unsigned long long )ph.sampling );
                        for( int k = 0; k < ph.sampling; k++ ) {
                            const unsigned long long o = o0 + ( unsigned long long )k;
                            if( o >= ( unsigned long long )ph.cap ) break;
                            for( int d = 0; d < ph.ndim; d++ ) ph.ph_pos[d * ph.cap + o] = ph.pos[d * n + p];
                            ph.ph_mom[o] = pg * px * inv;
                            ph.ph_mom[ph.cap + o] = pg * py * inv;
                            ph.ph_mom[2 * ph.cap + o] = pg * pz * inv;
                            ph.ph_w[o] = w[p] * ( 1.0 / ph.sampling );
                            ph.ph_chi[o] = pchi;
                            ph.ph_tau[o] = -1.0;
                        }
                        i_photon++;
                    } else {
                        rad += w[p] * ( g - sqrt( 1.0 + px * px + py * py + pz * pz ) );
                    }
                    nem++;
                    tp = -1.0;
                }
                it++;
                local_time += emission_time;
            } else if( chi <= t.min_disc && tp <= eps_tau && chi > t.min_cont ) {
                emission_time = dt - local_time;
                const double aa = 1.0 + 4.8 * ( 1.0 + chi ) * log( 1.0 + 1.7 * chi ) + 2.44 * chi * chi;
                const double e = ( 1.0 / cbrt( aa * aa ) ) * emission_time * chi * chi * t.factor_classical;
                const double tmp = e * g / ( g * g - 1.0 );
                px -= tmp * px;
                py -= tmp * py;
                pz -= tmp * pz;
                rad += w[p] * ( g - sqrt( 1.0 + px * px + py * py + pz * pz ) );
                local_time = dt;
            } else {
                local_time = dt;
            }
        }
        mom[p] = px;
        mom[n + p] = py;
        mom[2 * n + p] = pz;
        tau[p] = tp;
        // chi of the final momentum (RadiationMonteCarlo.cpp:642-655)
        if( chi_out ) chi_out[p] = particle_chi64( fabs( qm2 ) * t.inv_es, px, py, pz, Ex, Ey, Ez, Bx, By, Bz );
    }
    if constexpr( F32 ) {
        const bool active = p < n;
        const int64_t q = active ? p : 0;
        double px = 0.0, py = 0.0, pz = 0.0;
        float E3[3] = { 0.0f, 0.0f, 0.0f }, B3[3] = { 0.0f, 0.0f, 0.0f }, tp = 0.0f;
        if( active ) {
            px = mom[q];
            py = mom[n + q];
            pz = mom[2 * n + q];
            for( int c = 0; c < 3; c++ ) {
                E3[c] = ( float )Ep[c * n + q];
                B3[c] = ( float )Bp[c * n + q];
            }
            tp = ( float )tau[q];
        }
        uint32_t rs = rng_init( seed, first_id + ( uint32_t )q, step );
        double xp[3] = { 0.0, 0.0, 0.0 };
        for( int d = 0; ph.count && active && d < ph.ndim; d++ ) xp[d] = ph.pos[d * n + q];
        mc_pass_f32<H, double>( t, m, use_mlp, sw, active, dt, qm2, E3, B3, px, py, pz, tp, rs, w[q], rad, nem, ph, xp );
        if( active ) {
            mom[p] = px;
            mom[n + p] = py;
            mom[2 * n + p] = pz;
            tau[p] = ( double )tp;
            if( chi_out )
                chi_out[p] = particle_chi64( fabs( qm2 ) * t.inv_es, px, py, pz, E3[0], E3[1], E3[2], B3[0], B3[1], B3[2] );
        }
    }
    // block reduction of the tallies
    __shared__ double srad[32];
    __shared__ unsigned long long snem[32];
    for( int o = 16; o > 0; o >>= 1 ) {
        rad += __shfl_down_sync( 0xffffffffu, rad, o );
        nem += __shfl_down_sync( 0xffffffffu, nem, o );
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if( lane == 0 ) { srad[warp] = rad; snem[warp] = nem; }
    __syncthreads();
    if( threadIdx.x == 0 ) {
        double r = 0.0;
        unsigned long long e = 0;
        for( int k = 0; k < ( int )( blockDim.x >> 5 ); k++ ) { r += srad[k]; e += snem[k]; }
        if( r != 0.0 ) atomicAdd( radiated, r );
        if( e ) atomicAdd( n_emit, e );
    }
}

// PusherPhoton::operator() (src/Pusher/PusherPhoton.cpp:30-85): x += dt p / |p|.
__global__ void k_push_photons( int ndim, int64_t n, double dt, double *__restrict__ pos,
                                const double *__restrict__ mom, double *__restrict__ invgf )
{
    const int64_t p = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x;
    if( p >= n ) return;
    const double px = mom[p], py = mom[n + p], pz = mom[2 * n + p];
    const double inv = 1.0 / sqrt( px * px + py * py + pz * pz );
    if( invgf ) invgf[p] = inv;
    pos[p] += dt * px * inv;
    if( ndim > 1 ) pos[n + p] += dt * py * inv;
    if( ndim > 2 ) pos[2 * n + p] += dt * pz * inv;
}

// The pass over a resident 2D mixed-form species, one block per tile: each
// particle's E and B_m come from an order-2 gather of the global field arrays (the
// gather of the step kernel, here from global memory), then mc_pass_f32 updates its
// momentum and optical depth in place.  The random stream of the particle in slot o at
// step k is (seed, o, k).  Runs before the step, as Radiate before the push in
// Species::dynamics (Species.cpp:583-640).
__device__ __forceinline__ void bspl2( float x, float &c0, float &c1, float &c2 )
{
    c0 = 0.5f * ( 0.5f - x ) * ( 0.5f - x );
    c1 = 0.75f - x * x;
    c2 = 0.5f * ( 0.5f + x ) * ( 0.5f + x );
}

__device__ __forceinline__ float gather2( const float *__restrict__ F, int ny, int bx, int by, const float *cx,
                                          const float *cy )
{
    float r = 0.0f;
#pragma unroll
    for( int a = 0; a < 3; a++ ) {
        const float *row = F + ( int64_t )( bx + a ) * ny + by;
        r = fmaf( cx[a], cy[0] * __ldg( row ) + cy[1] * __ldg( row + 1 ) + cy[2] * __ldg( row + 2 ), r );
    }
    return r;
}

template <int H, bool PH>
__global__ void __launch_bounds__( 128 ) k_radiate_resident( RadTab t, MlpView m, int use_mlp, ResidentRad r,
                                                             int64_t nslots )
{
    __shared__ MlpShared<H == 0 ? 4 : H> sw;
    if constexpr( H > 0 ) {
        mlp_stage<H, true>( m, sw );
        __syncthreads();
    }
    const uint32_t step = ( uint32_t )*r.step;
    const int nyp = r.np[1], nyd = nyp + 1;
    // macro-photons of the species, when it has a photon store
    PhotonOut ph{};
    if( PH && r.ph_count ) {
        ph.ndim = 2;
        ph.dx[0] = r.dx[0];
        ph.dx[1] = r.dx[1];
        ph.sampling = r.ph_sampling;
        ph.max_emissions = r.ph_max_emissions;
        ph.threshold = r.ph_threshold;
        ph.cap = r.ph_cap;
        ph.count = r.ph_count;
        ph.ph_pos = r.ph_pos;
        ph.ph_mom = r.ph_mom;
        ph.ph_w = r.ph_w;
        ph.ph_chi = r.ph_chi;
        ph.ph_tau = r.ph_tau;
    }
    double rad = 0.0;
    unsigned long long nem = 0;
    // one thread per buffer slot (all tiles' segments, holes included), so that a few
    // dense tiles still spread over the whole GPU; a slot's tile is found by a binary
    // search of the segment starts
    for( int64_t o0 = ( int64_t )blockIdx.x * blockDim.x; o0 < nslots; o0 += ( int64_t )gridDim.x * blockDim.x ) {
        const int64_t o = o0 + threadIdx.x;
        bool active = false;
        if( o < nslots ) {
            int lo = 0, hi = r.ntiles - 1; // last tile whose segment starts at or before o
            while( lo < hi ) {
                const int mid = ( lo + hi + 1 ) >> 1;
                if( r.seg_start[mid] <= o ) lo = mid;
                else hi = mid - 1;
            }
            active = o - r.seg_start[lo] < r.count[lo];
        }
        float px = 0.0f, py = 0.0f, pz = 0.0f;
        float E3[3] = { 0.0f, 0.0f, 0.0f }, B3[3] = { 0.0f, 0.0f, 0.0f }, tp = 0.0f, wq = 0.0f;
        int xn[2] = { 0, 0 };            // the particle's node and offset: where its photons start
        float xo[2] = { 0.0f, 0.0f };
        if( active ) {
            const unsigned k = r.key[o];
            const int gx = ( int )( k >> 16 ), gy = ( int )( k & 65535u );
            const float dxl = r.d[0][o], dyl = r.d[1][o];
            xn[0] = gx;
            xn[1] = gy;
            xo[0] = dxl;
            xo[1] = dyl;
            float cpx[3], cpy[3], cdx[3], cdy[3];
            bspl2( dxl, cpx[0], cpx[1], cpx[2] );
            bspl2( dyl, cpy[0], cpy[1], cpy[2] );
            const int sx = dxl >= 0.0f ? 1 : 0, sy = dyl >= 0.0f ? 1 : 0;
            bspl2( dxl + 0.5f - ( float )sx, cdx[0], cdx[1], cdx[2] );
            bspl2( dyl + 0.5f - ( float )sy, cdy[0], cdy[1], cdy[2] );
            // primal node gx sits at array index gx + 2; the stencil starts one node below
            const int bxp = gx + 1, byp = gy + 1, bxd = gx + 1 + sx, byd = gy + 1 + sy;
            // Ex(d,p) Ey(p,d) Ez(p,p) Bx(p,d) By(d,p) Bz(d,d)
            E3[0] = gather2( r.E[0], nyp, bxd, byp, cdx, cpy );
            E3[1] = gather2( r.E[1], nyd, bxp, byd, cpx, cdy );
            E3[2] = gather2( r.E[2], nyp, bxp, byp, cpx, cpy );
            B3[0] = gather2( r.Bm[0], nyd, bxp, byd, cpx, cdy );
            B3[1] = gather2( r.Bm[1], nyp, bxd, byp, cdx, cpy );
            B3[2] = gather2( r.Bm[2], nyd, bxd, byd, cdx, cdy );
            px = r.p[0][o];
            py = r.p[1][o];
            pz = r.p[2][o];
            tp = r.tau[o];
            wq = r.w[o];
        }
        uint32_t rs = rng_init( r.seed, ( uint32_t )o, step );
        mc_pass_f32<H, float, PH>( t, m, use_mlp, sw, active, r.dt, r.qm2, E3, B3, px, py, pz, tp, rs, ( double )wq, rad,
                                   nem, ph, nullptr, xn, xo );
        if( active ) {
            r.p[0][o] = px;
            r.p[1][o] = py;
            r.p[2][o] = pz;
            r.tau[o] = tp;
        }
    }
    __shared__ double srad[4];
    __shared__ unsigned long long snem[4];
    for( int k = 16; k > 0; k >>= 1 ) {
        rad += __shfl_down_sync( 0xffffffffu, rad, k );
        nem += __shfl_down_sync( 0xffffffffu, nem, k );
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if( lane == 0 ) {
        srad[warp] = rad;
        snem[warp] = nem;
    }
    __syncthreads();
    if( threadIdx.x == 0 ) {
        double a = 0.0;
        unsigned long long e = 0;
        for( int k = 0; k < ( int )( blockDim.x >> 5 ); k++ ) {
            a += srad[k];
            e += snem[k];
        }
        if( a != 0.0 ) atomicAdd( r.radiated, a );
        if( e ) atomicAdd( r.emissions, e );
    }
}

// ---- MLP training ------------------------------------------------------------
// Samples: log10 chi uniform in [lmin, lmin + lspan], xi uniform in [0, 1) (input
// mlp_xi_input(xi));
// target = log10(table photon chi / chi) / out_scale.
__global__ void k_mlp_samples( RadTab t, int B, float lmin, float lspan, float out_scale, uint32_t seed,
                               uint32_t step, float *__restrict__ X, float *__restrict__ Y )
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if( b >= B ) return;
    uint32_t rs = rng_init( seed, ( uint32_t )b, step );
    const double l = lmin + lspan * rng_uniform( rs );
    const double xi = rng_uniform( rs );
    const double chi = pow( 10.0, l );
    const double pc = tab_photon_chi( t, chi, xi );
    X[2 * b] = 2.0f * ( float )( ( l - lmin ) / lspan ) - 1.0f;
    X[2 * b + 1] = mlp_xi_input( ( float )xi );
    Y[b] = ( float )( log10( pc / chi ) / out_scale );
}

// Forward + backward per sample for the mean-squared loss; stores h1, h2 and the
// deltas of both hidden layers for the weight-gradient reduction.
__global__ void k_mlp_fwd_bwd( MlpView m, int B, const float *__restrict__ X, const float *__restrict__ Y,
                               float *__restrict__ H1, float *__restrict__ H2, float *__restrict__ D1,
                               float *__restrict__ D2, float *__restrict__ D3, float *__restrict__ loss )
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    const int H = m.H;
    float l = 0.0f;
    if( b < B ) {
        float h1[MLP_MAX_H], h2[MLP_MAX_H], d2[MLP_MAX_H];
        const float u0 = X[2 * b], u1 = X[2 * b + 1];
        const float y = mlp_forward( m, u0, u1, h1, h2 );
        const float e = y - Y[b];
        l = e * e;
        const float d3 = 2.0f * e / ( float )B;
        D3[b] = d3;
        for( int i = 0; i < H; i++ ) {
            d2[i] = m.W3[i] * d3 * ( 1.0f - h2[i] * h2[i] );
            H1[( int64_t )b * H + i] = h1[i];
            H2[( int64_t )b * H + i] = h2[i];
            D2[( int64_t )b * H + i] = d2[i];
        }
        for( int j = 0; j < H; j++ ) {
            float a = 0.0f;
            for( int i = 0; i < H; i++ ) a = fmaf( m.W2[i * H + j], d2[i], a );
            D1[( int64_t )b * H + j] = a * ( 1.0f - h1[j] * h1[j] );
        }
    }
    for( int o = 16; o > 0; o >>= 1 ) l += __shfl_down_sync( 0xffffffffu, l, o );
    if( ( threadIdx.x & 31 ) == 0 && loss ) atomicAdd( loss, l / ( float )B );
}

// One thread per parameter: the gradient as a sum over the batch (deterministic order).
__global__ void k_mlp_grads( int H, int B, const float *__restrict__ X, const float *__restrict__ H1,
                             const float *__restrict__ H2, const float *__restrict__ D1, const float *__restrict__ D2,
                             const float *__restrict__ D3, float *__restrict__ G )
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int P = mlp_nparams( H );
    if( k >= P ) return;
    // layout: W1[H*2] b1[H] W2[H*H] b2[H] W3[H] b3[1]
    float acc = 0.0f;
    if( k < 2 * H ) {
        const int i = k / 2, c = k % 2;
        for( int b = 0; b < B; b++ ) acc = fmaf( D1[( int64_t )b * H + i], X[2 * b + c], acc );
    } else if( k < 3 * H ) {
        const int i = k - 2 * H;
        for( int b = 0; b < B; b++ ) acc += D1[( int64_t )b * H + i];
    } else if( k < 3 * H + H * H ) {
        const int q = k - 3 * H, i = q / H, j = q % H;
        for( int b = 0; b < B; b++ ) acc = fmaf( D2[( int64_t )b * H + i], H1[( int64_t )b * H + j], acc );
    } else if( k < 4 * H + H * H ) {
        const int i = k - 3 * H - H * H;
        for( int b = 0; b < B; b++ ) acc += D2[( int64_t )b * H + i];
    } else if( k < 5 * H + H * H ) {
        const int j = k - 4 * H - H * H;
        for( int b = 0; b < B; b++ ) acc = fmaf( D3[b], H2[( int64_t )b * H + j], acc );
    } else {
        for( int b = 0; b < B; b++ ) acc += D3[b];
    }
    G[k] = acc;
}

// Adam (Kingma & Ba 2015) with bias correction.
__global__ void k_adam( int P, float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m1,
                        float *__restrict__ m2, float lr, float b1, float b2, float eps, int t )
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if( k >= P ) return;
    const float gk = g[k];
    const float a = b1 * m1[k] + ( 1.0f - b1 ) * gk;
    const float c = b2 * m2[k] + ( 1.0f - b2 ) * gk * gk;
    m1[k] = a;
    m2[k] = c;
    const float ah = a / ( 1.0f - powf( b1, ( float )t ) ), ch = c / ( 1.0f - powf( b2, ( float )t ) );
    w[k] -= lr * ah / ( sqrtf( ch ) + eps );
}

// Validation: per (chi bin, xi bin), the largest |log10 mlp - log10 table| over a
// regular sub-grid of the bin.
__global__ void k_mlp_validate( RadTab t, MlpView m, int per_bin, float *__restrict__ err )
{
    const int bin = blockIdx.x;
    const int bc = bin / m.nbx, bx = bin % m.nbx;
    float e = 0.0f;
    for( int s = threadIdx.x; s < per_bin * per_bin; s += blockDim.x ) {
        const int sc = s / per_bin, sx = s % per_bin;
        const double l = m.lmin + m.lspan * ( bc + ( sc + 0.5 ) / per_bin ) / m.nbc;
        const double xi = ( bx + ( sx + 0.5 ) / per_bin ) / m.nbx;
        const double chi = pow( 10.0, l );
        const double a = log10( mlp_photon_chi( m, chi, xi ) ), b = log10( tab_photon_chi( t, chi, xi ) );
        e = fmaxf( e, ( float )fabs( a - b ) );
    }
    for( int o = 16; o > 0; o >>= 1 ) e = fmaxf( e, __shfl_down_sync( 0xffffffffu, e, o ) );
    __shared__ float se[32];
    if( ( threadIdx.x & 31 ) == 0 ) se[threadIdx.x >> 5] = e;
    __syncthreads();
    if( threadIdx.x == 0 ) {
        float r = 0.0f;
        for( int k = 0; k < ( int )( blockDim.x >> 5 ); k++ ) r = fmaxf( r, se[k] );
        err[bin] = r;
    }
}

} // namespace
} // namespace sg

using namespace sg;

struct sg_rad_tables {
    RadTab t;
    double *mem = nullptr;
    float *memf = nullptr; // FP32 copies of the tables
    int fp32 = 0;          // Monte-Carlo arithmetic: 0 FP64, 1 FP32 (sg_rad_tables_set_fp32_math)
};

struct sg_mlp {
    int H = 64;
    float *params = nullptr; // device, nparams
    float *m1 = nullptr, *m2 = nullptr, *grad = nullptr;
    int adam_t = 0;
    float lmin = -4.0f, lspan = 7.0f, out_scale = 8.0f;
    int *mask = nullptr; // device
    int nbc = 0, nbx = 0;
    float *scratch = nullptr;
    int scratch_B = 0;
};

namespace {

MlpView view( const sg_mlp *m )
{
    MlpView v;
    v.H = m->H;
    const int H = m->H;
    v.W1 = m->params;
    v.b1 = v.W1 + 2 * H;
    v.W2 = v.b1 + H;
    v.b2 = v.W2 + H * H;
    v.W3 = v.b2 + H;
    v.b3 = v.W3 + H;
    v.lmin = m->lmin;
    v.lspan = m->lspan;
    v.out_scale = m->out_scale;
    v.mask = m->mask;
    v.nbc = m->nbc;
    v.nbx = m->nbx;
    return v;
}

int ensure_scratch( sg_mlp *m, int B )
{
    if( m->scratch_B >= B ) return SG_OK;
    release( m->scratch );
    m->scratch = nullptr;
    const size_t floats = ( size_t )B * ( 4 * m->H + 4 ) + 64;
    SG_CUDA_TRY( cudaMalloc( &m->scratch, floats * sizeof( float ) ) );
    m->scratch_B = B;
    return SG_OK;
}

} // namespace

namespace sg {
namespace {
// The Monte-Carlo kernel for the tables' arithmetic and the network's width.
using McKernel = void ( * )( RadTab, MlpView, int, int64_t, double, double, double *, const double *, double *,
                             double *, const double *, const double *, uint32_t, uint32_t, uint32_t, double *,
                             unsigned long long *, PhotonOut );
template <bool F32>
McKernel mc_kernel_for( int H )
{
    if( H == 64 ) return k_monte_carlo<F32, 64>;
    if( H == 32 ) return k_monte_carlo<F32, 32>;
    if( H == 16 ) return k_monte_carlo<F32, 16>;
    return k_monte_carlo<F32, 0>;
}
} // namespace
} // namespace sg

namespace sg {
int launch_radiate_resident( const sg_rad_tables *T, const sg_mlp *mlp, const ResidentRad &r, cudaStream_t st )
{
    if( mlp ) SG_REQUIRE( mlp->mask != nullptr, "the network has not been validated (sg_mlp_validate)" );
    MlpView v{};
    if( mlp ) v = view( mlp );
    const int H = mlp ? v.H : 0;
    const unsigned blocks = ( unsigned )std::min<int64_t>( ( r.nslots + 127 ) / 128, 152 * 64 );
    if( r.nslots <= 0 ) return SG_OK;
    // the photon output is a separate instance, so that a species without one keeps the
    // registers of the plain pass
    if( r.ph_count ) {
        if( H == 64 ) k_radiate_resident<64, true><<<blocks, 128, 0, st>>>( T->t, v, 1, r, r.nslots );
        else if( H == 32 ) k_radiate_resident<32, true><<<blocks, 128, 0, st>>>( T->t, v, 1, r, r.nslots );
        else if( H == 16 ) k_radiate_resident<16, true><<<blocks, 128, 0, st>>>( T->t, v, 1, r, r.nslots );
        else k_radiate_resident<0, true><<<blocks, 128, 0, st>>>( T->t, v, mlp ? 1 : 0, r, r.nslots );
    } else {
        if( H == 64 ) k_radiate_resident<64, false><<<blocks, 128, 0, st>>>( T->t, v, 1, r, r.nslots );
        else if( H == 32 ) k_radiate_resident<32, false><<<blocks, 128, 0, st>>>( T->t, v, 1, r, r.nslots );
        else if( H == 16 ) k_radiate_resident<16, false><<<blocks, 128, 0, st>>>( T->t, v, 1, r, r.nslots );
        else k_radiate_resident<0, false><<<blocks, 128, 0, st>>>( T->t, v, mlp ? 1 : 0, r, r.nslots );
    }
    SG_LAUNCH_CHECK( "k_radiate_resident" );
    return SG_OK;
}
} // namespace sg

extern "C" {


int sg_rad_tables_create( const double *integ, int n_integ, double integ_min, double integ_max, const double *xi,
                          int n_chi, int n_ph, double xi_min, double xi_max, const double *axis1_min,
                          const double *factors, sg_rad_tables **out )
{
    SG_REQUIRE( integ && xi && axis1_min && factors && out, "NULL argument" );
    SG_REQUIRE( n_integ >= 2 && n_chi >= 2 && n_ph >= 2, "tables need at least two points per axis" );
    SG_REQUIRE( integ_min > 0 && integ_max > integ_min && xi_min > 0 && xi_max > xi_min, "bad table range" );
    sg_rad_tables *T = new sg_rad_tables();
    const size_t n = ( size_t )n_integ + ( size_t )n_chi * n_ph + n_chi;
    cudaError_t e = cudaMalloc( &T->mem, n * sizeof( double ) );
    if( e != cudaSuccess ) { delete T; return set_error( SG_ERR_NOMEM, "cannot allocate the radiation tables" ); }
    double *d_integ = T->mem, *d_xi = d_integ + n_integ, *d_ax = d_xi + ( size_t )n_chi * n_ph;
    if( cudaMemcpy( d_integ, integ, n_integ * sizeof( double ), cudaMemcpyHostToDevice ) != cudaSuccess ||
        cudaMemcpy( d_xi, xi, ( size_t )n_chi * n_ph * sizeof( double ), cudaMemcpyHostToDevice ) != cudaSuccess ||
        cudaMemcpy( d_ax, axis1_min, n_chi * sizeof( double ), cudaMemcpyHostToDevice ) != cudaSuccess ) {
        release( T->mem );
        delete T;
        return set_error( SG_ERR_CUDA, "cannot copy the radiation tables" );
    }
    RadTab &t = T->t;
    t.integ = d_integ;
    t.n_integ = n_integ;
    t.integ_l0 = std::log10( integ_min );
    t.integ_d = ( std::log10( integ_max ) - t.integ_l0 ) / ( n_integ - 1 );
    t.integ_id = 1.0 / t.integ_d;
    t.xi = d_xi;
    t.n_chi = n_chi;
    t.n_ph = n_ph;
    t.xi_l0 = std::log10( xi_min );
    t.xi_d = ( std::log10( xi_max ) - t.xi_l0 ) / ( n_chi - 1 );
    t.xi_id = 1.0 / t.xi_d;
    t.inv_nph_m1 = 1.0 / ( n_ph - 1 );
    t.axis1_min = d_ax;
    t.factor_dNph_dt = factors[0];
    t.factor_classical = factors[1];
    t.inv_es = factors[2];
    t.min_cont = factors[3];
    t.min_disc = factors[4];
    {
        std::vector<float> hf( n );
        for( int i = 0; i < n_integ; i++ ) hf[i] = ( float )integ[i];
        for( size_t i = 0; i < ( size_t )n_chi * n_ph; i++ ) hf[n_integ + i] = ( float )xi[i];
        for( int i = 0; i < n_chi; i++ ) hf[n_integ + ( size_t )n_chi * n_ph + i] = ( float )axis1_min[i];
        if( cudaMalloc( &T->memf, n * sizeof( float ) ) != cudaSuccess ||
            cudaMemcpy( T->memf, hf.data(), n * sizeof( float ), cudaMemcpyHostToDevice ) != cudaSuccess ) {
            release( T->mem );
            release( T->memf );
            delete T;
            return set_error( SG_ERR_NOMEM, "cannot allocate the FP32 radiation tables" );
        }
        t.integf = T->memf;
        t.xif = T->memf + n_integ;
        t.axis1_minf = T->memf + n_integ + ( size_t )n_chi * n_ph;
    }
    *out = T;
    return SG_OK;
}

int sg_rad_tables_set_fp32_math( sg_rad_tables *T, int on )
{
    SG_REQUIRE( T, "NULL tables" );
    T->fp32 = on ? 1 : 0;
    return SG_OK;
}

int sg_rad_tables_destroy( sg_rad_tables *T )
{
    if( !T ) return SG_OK;
    release( T->mem );
    release( T->memf );
    delete T;
    return SG_OK;
}

int sg_rad_photon_chi( const sg_rad_tables *T, int64_t n, const double *chi, const double *xi, double *out,
                       sg_stream_t stream )
{
    SG_REQUIRE( T && chi && xi && out, "NULL argument" );
    if( n <= 0 ) return SG_OK;
    k_photon_chi<<<grid_for( n, 256 ), 256, 0, as_stream( stream )>>>( T->t, n, chi, xi, out );
    SG_LAUNCH_CHECK( "k_photon_chi" );
    return SG_OK;
}

int sg_rad_production_yield( const sg_rad_tables *T, int64_t n, const double *chi, const double *gamma, double *out,
                             sg_stream_t stream )
{
    SG_REQUIRE( T && chi && gamma && out, "NULL argument" );
    if( n <= 0 ) return SG_OK;
    k_yield<<<grid_for( n, 256 ), 256, 0, as_stream( stream )>>>( T->t, n, chi, gamma, out );
    SG_LAUNCH_CHECK( "k_yield" );
    return SG_OK;
}

int sg_rad_monte_carlo( const sg_rad_tables *T, const sg_mlp *mlp, int64_t n, double dt, double mass,
                        double charge, double *mom, const double *weight, double *tau, double *chi_out,
                        const double *Epart, const double *Bpart, uint32_t seed, uint32_t first_id, uint32_t step,
                        double *radiated, unsigned long long *n_emissions, sg_stream_t stream )
{
    SG_REQUIRE( T && mom && weight && tau && Epart && Bpart && radiated && n_emissions, "NULL argument" );
    SG_REQUIRE( mass > 0.0, "mass must be positive" );
    if( mlp ) SG_REQUIRE( mlp->mask != nullptr, "the network has not been validated (sg_mlp_validate)" );
    if( n <= 0 ) return SG_OK;
    const double oom = 1.0 / mass;
    MlpView v{};
    if( mlp ) v = view( mlp );
    const int H = mlp ? v.H : 0;
    McKernel kern = T->fp32 ? mc_kernel_for<true>( H ) : mc_kernel_for<false>( H );
    kern<<<grid_for( n, 256 ), 256, 0, as_stream( stream )>>>( T->t, v, mlp ? 1 : 0, n, dt, charge * oom * oom, mom, weight,
                                                                tau, chi_out, Epart, Bpart, seed, first_id, step, radiated,
                                                                n_emissions, PhotonOut{} );
    SG_LAUNCH_CHECK( "k_monte_carlo" );
    return SG_OK;
}

int sg_rad_monte_carlo_photons( const sg_rad_tables *T, const sg_mlp *mlp, int ndim, int64_t n, double dt,
                                double mass, double charge, const double *pos, double *mom, const double *weight,
                                double *tau, double *chi_out, const double *Epart, const double *Bpart, uint32_t seed,
                                uint32_t first_id, uint32_t step, int sampling, double gamma_threshold,
                                int max_emissions, int64_t photon_capacity, double *ph_pos, double *ph_mom,
                                double *ph_weight, double *ph_chi, double *ph_tau, unsigned long long *n_photons,
                                double *radiated, unsigned long long *n_emissions, sg_stream_t stream )
{
    SG_REQUIRE( T && pos && mom && weight && tau && Epart && Bpart && radiated && n_emissions && n_photons,
                "NULL argument" );
    SG_REQUIRE( ndim >= 1 && ndim <= 3, "ndim must be 1, 2 or 3" );
    SG_REQUIRE( mass > 0.0, "mass must be positive" );
    SG_REQUIRE( sampling >= 1 && max_emissions >= 1, "sampling and max_emissions must be at least 1" );
    SG_REQUIRE( photon_capacity >= 0, "photon_capacity < 0" );
    if( photon_capacity > 0 ) SG_REQUIRE( ph_pos && ph_mom && ph_weight && ph_chi && ph_tau, "NULL photon array" );
    if( mlp ) SG_REQUIRE( mlp->mask != nullptr, "the network has not been validated (sg_mlp_validate)" );
    if( n <= 0 ) return SG_OK;
    const double oom = 1.0 / mass;
    MlpView v{};
    if( mlp ) v = view( mlp );
    PhotonOut ph{ pos, ndim, sampling, max_emissions, gamma_threshold, photon_capacity, n_photons,
                  ph_pos, ph_mom, ph_weight, ph_chi, ph_tau };
    const int H = mlp ? v.H : 0;
    McKernel kern = T->fp32 ? mc_kernel_for<true>( H ) : mc_kernel_for<false>( H );
    kern<<<grid_for( n, 256 ), 256, 0, as_stream( stream )>>>( T->t, v, mlp ? 1 : 0, n, dt, charge * oom * oom, mom, weight,
                                                                tau, chi_out, Epart, Bpart, seed, first_id, step, radiated,
                                                                n_emissions, ph );
    SG_LAUNCH_CHECK( "k_monte_carlo" );
    return SG_OK;
}

int sg_push_photons( int ndim, int64_t n, double dt, double *pos, const double *mom, double *invgf,
                     sg_stream_t stream )
{
    SG_REQUIRE( ndim >= 1 && ndim <= 3, "ndim must be 1, 2 or 3" );
    if( n <= 0 ) return SG_OK;
    SG_REQUIRE( pos && mom, "NULL argument" );
    k_push_photons<<<grid_for( n, 256 ), 256, 0, as_stream( stream )>>>( ndim, n, dt, pos, mom, invgf );
    SG_LAUNCH_CHECK( "k_push_photons" );
    return SG_OK;
}

int sg_mlp_create( int hidden, uint32_t seed, double log10_chi_min, double log10_chi_max, sg_mlp **out )
{
    SG_REQUIRE( out, "NULL argument" );
    SG_REQUIRE( hidden >= 4 && hidden <= MLP_MAX_H, "hidden width must be in [4, %d]", MLP_MAX_H );
    SG_REQUIRE( log10_chi_max > log10_chi_min, "empty chi range" );
    sg_mlp *m = new sg_mlp();
    m->H = hidden;
    m->lmin = ( float )log10_chi_min;
    m->lspan = ( float )( log10_chi_max - log10_chi_min );
    const int P = mlp_nparams( hidden );
    std::vector<float> h( P, 0.0f );
    // Xavier-uniform weights from a hashed counter, zero biases
    auto u = [&]( uint32_t k ) { return ( fmix32( seed * 0x9e3779b9u + k ) >> 8 ) * ( 1.0f / 16777216.0f ) * 2.0f - 1.0f; };
    const int H = hidden;
    for( int k = 0; k < 2 * H; k++ ) h[k] = u( k ) * std::sqrt( 6.0f / ( 2 + H ) );
    for( int k = 0; k < H * H; k++ ) h[3 * H + k] = u( 100000 + k ) * std::sqrt( 6.0f / ( 2 * H ) );
    for( int k = 0; k < H; k++ ) h[4 * H + H * H + k] = u( 200000 + k ) * std::sqrt( 6.0f / ( H + 1 ) );
    cudaError_t e = cudaMalloc( &m->params, 4 * ( size_t )P * sizeof( float ) );
    if( e != cudaSuccess ) { delete m; return set_error( SG_ERR_NOMEM, "cannot allocate the network" ); }
    m->m1 = m->params + P;
    m->m2 = m->m1 + P;
    m->grad = m->m2 + P;
    cudaMemcpy( m->params, h.data(), P * sizeof( float ), cudaMemcpyHostToDevice );
    cudaMemset( m->m1, 0, 3 * ( size_t )P * sizeof( float ) );
    if( cudaGetLastError() != cudaSuccess ) { release( m->params ); delete m; return set_error( SG_ERR_CUDA, "network init failed" ); }
    *out = m;
    return SG_OK;
}

int sg_mlp_destroy( sg_mlp *m )
{
    if( !m ) return SG_OK;
    release( m->params );
    release( m->mask );
    release( m->scratch );
    delete m;
    return SG_OK;
}

int sg_mlp_nparams( const sg_mlp *m, int *n )
{
    SG_REQUIRE( m && n, "NULL argument" );
    *n = mlp_nparams( m->H );
    return SG_OK;
}

int sg_mlp_get_params( const sg_mlp *m, float *host )
{
    SG_REQUIRE( m && host, "NULL argument" );
    SG_CUDA_TRY( cudaMemcpy( host, m->params, mlp_nparams( m->H ) * sizeof( float ), cudaMemcpyDeviceToHost ) );
    return SG_OK;
}

int sg_mlp_set_params( sg_mlp *m, const float *host )
{
    SG_REQUIRE( m && host, "NULL argument" );
    SG_CUDA_TRY( cudaMemcpy( m->params, host, mlp_nparams( m->H ) * sizeof( float ), cudaMemcpyHostToDevice ) );
    return SG_OK;
}

int sg_mlp_gradients( sg_mlp *m, int B, const float *inputs, const float *targets, float *grad, float *loss )
{
    SG_REQUIRE( m && inputs && targets && grad && loss, "NULL argument" );
    SG_REQUIRE( B > 0, "empty batch" );
    int r = ensure_scratch( m, B );
    if( r ) return r;
    const int H = m->H, P = mlp_nparams( H );
    float *X = m->scratch, *Y = X + 2 * ( size_t )B, *H1 = Y + B, *H2 = H1 + ( size_t )B * H, *D1 = H2 + ( size_t )B * H;
    float *D2 = D1 + ( size_t )B * H, *D3 = D2 + ( size_t )B * H, *L = D3 + B;
    SG_CUDA_TRY( cudaMemcpy( X, inputs, 2 * ( size_t )B * sizeof( float ), cudaMemcpyHostToDevice ) );
    SG_CUDA_TRY( cudaMemcpy( Y, targets, ( size_t )B * sizeof( float ), cudaMemcpyHostToDevice ) );
    SG_CUDA_TRY( cudaMemset( L, 0, sizeof( float ) ) );
    k_mlp_fwd_bwd<<<grid_for( B, 128 ), 128>>>( view( m ), B, X, Y, H1, H2, D1, D2, D3, L );
    k_mlp_grads<<<grid_for( P, 128 ), 128>>>( H, B, X, H1, H2, D1, D2, D3, m->grad );
    SG_LAUNCH_CHECK( "k_mlp_grads" );
    SG_CUDA_TRY( cudaMemcpy( grad, m->grad, P * sizeof( float ), cudaMemcpyDeviceToHost ) );
    SG_CUDA_TRY( cudaMemcpy( loss, L, sizeof( float ), cudaMemcpyDeviceToHost ) );
    return SG_OK;
}

int sg_mlp_train( sg_mlp *m, const sg_rad_tables *T, int steps, int B, float lr, uint32_t seed, float *final_loss,
                  sg_stream_t stream )
{
    SG_REQUIRE( m && T, "NULL argument" );
    SG_REQUIRE( steps >= 0 && B > 0, "bad training sizes" );
    int r = ensure_scratch( m, B );
    if( r ) return r;
    cudaStream_t st = as_stream( stream );
    const int H = m->H, P = mlp_nparams( H );
    float *X = m->scratch, *Y = X + 2 * ( size_t )B, *H1 = Y + B, *H2 = H1 + ( size_t )B * H, *D1 = H2 + ( size_t )B * H;
    float *D2 = D1 + ( size_t )B * H, *D3 = D2 + ( size_t )B * H, *L = D3 + B;
    for( int s = 0; s < steps; s++ ) {
        k_mlp_samples<<<grid_for( B, 256 ), 256, 0, st>>>( T->t, B, m->lmin, m->lspan, m->out_scale, seed, ( uint32_t )s, X, Y );
        if( s == steps - 1 ) SG_CUDA_TRY( cudaMemsetAsync( L, 0, sizeof( float ), st ) );
        k_mlp_fwd_bwd<<<grid_for( B, 128 ), 128, 0, st>>>( view( m ), B, X, Y, H1, H2, D1, D2, D3, s == steps - 1 ? L : nullptr );
        k_mlp_grads<<<grid_for( P, 128 ), 128, 0, st>>>( H, B, X, H1, H2, D1, D2, D3, m->grad );
        m->adam_t++;
        k_adam<<<grid_for( P, 256 ), 256, 0, st>>>( P, m->params, m->grad, m->m1, m->m2, lr, 0.9f, 0.999f, 1e-8f, m->adam_t );
        SG_LAUNCH_CHECK( "k_adam" );
    }
    if( final_loss ) {
        SG_CUDA_TRY( cudaMemcpyAsync( final_loss, L, sizeof( float ), cudaMemcpyDeviceToHost, st ) );
        SG_CUDA_TRY( cudaStreamSynchronize( st ) );
    }
    return SG_OK;
}

int sg_mlp_validate( sg_mlp *m, const sg_rad_tables *T, int n_chi_bins, int n_xi_bins, int per_bin, float tol,
                     float *err_out, int *n_masked )
{
    SG_REQUIRE( m && T, "NULL argument" );
    SG_REQUIRE( n_chi_bins > 0 && n_xi_bins > 0 && per_bin > 0, "bad validation grid" );
    const int nb = n_chi_bins * n_xi_bins;
    release( m->mask );
    m->mask = nullptr;
    SG_CUDA_TRY( cudaMalloc( &m->mask, nb * sizeof( int ) ) );
    m->nbc = n_chi_bins;
    m->nbx = n_xi_bins;
    float *d_err = nullptr;
    SG_CUDA_TRY( cudaMalloc( &d_err, nb * sizeof( float ) ) );
    k_mlp_validate<<<nb, 256>>>( T->t, view( m ), per_bin, d_err );
    SG_LAUNCH_CHECK( "k_mlp_validate" );
    std::vector<float> h( nb );
    SG_CUDA_TRY( cudaMemcpy( h.data(), d_err, nb * sizeof( float ), cudaMemcpyDeviceToHost ) );
    release( d_err );
    std::vector<int> mask( nb );
    int cnt = 0;
    for( int i = 0; i < nb; i++ ) {
        mask[i] = !( h[i] <= tol ); // NaN -> masked
        cnt += mask[i];
    }
    SG_CUDA_TRY( cudaMemcpy( m->mask, mask.data(), nb * sizeof( int ), cudaMemcpyHostToDevice ) );
    if( err_out ) std::copy( h.begin(), h.end(), err_out );
    if( n_masked ) *n_masked = cnt;
    return SG_OK;
}

int sg_mlp_photon_chi( const sg_mlp *m, int64_t n, const double *chi, const double *xi, double *out, sg_stream_t stream )
{
    SG_REQUIRE( m && chi && xi && out, "NULL argument" );
    if( n <= 0 ) return SG_OK;
    if( m->H != TC_H ) return sg_mlp_photon_chi_fp32( m, n, chi, xi, out, stream );
    const int64_t tiles = ( n + 31 ) / 32;
    const unsigned blocks = ( unsigned )std::min<int64_t>( ( tiles + 3 ) / 4, 152 * 8 );
    k_mlp_photon_chi_tc<<<blocks, 128, 0, as_stream( stream )>>>( view( m ), n, chi, xi, out );
    SG_LAUNCH_CHECK( "k_mlp_photon_chi_tc" );
    return SG_OK;
}

int sg_mlp_photon_chi_fp32( const sg_mlp *m, int64_t n, const double *chi, const double *xi, double *out,
                            sg_stream_t stream )
{
    SG_REQUIRE( m && chi && xi && out, "NULL argument" );
    if( n <= 0 ) return SG_OK;
    const unsigned blocks = ( unsigned )std::min<int64_t>( ( n + 255 ) / 256, 152 * 8 );
    if( m->H == 64 ) k_mlp_photon_chi_fast<64><<<blocks, 256, 0, as_stream( stream )>>>( view( m ), n, chi, xi, out );
    else if( m->H == 32 ) k_mlp_photon_chi_fast<32><<<blocks, 256, 0, as_stream( stream )>>>( view( m ), n, chi, xi, out );
    else if( m->H == 16 ) k_mlp_photon_chi_fast<16><<<blocks, 256, 0, as_stream( stream )>>>( view( m ), n, chi, xi, out );
    else k_mlp_photon_chi<<<grid_for( n, 128 ), 128, 0, as_stream( stream )>>>( view( m ), n, chi, xi, out );
    SG_LAUNCH_CHECK( "k_mlp_photon_chi" );
    return SG_OK;
}

} // extern "C"
