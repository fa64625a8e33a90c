// The simulation object: a whole periodic PIC timestep resident on one GPU.
//
// Layout in HBM
//   fields   one array per component in the reference's layout (ghost width
//            2, primal N+5 / dual N+6 points per dimension, x-major), in the
//            form's precision (FP64 or FP32): E, B, B_m, J.
//   tiles    the grid is cut into tiles (bins) of T cells per dimension; a
//            particle belongs to the tile of its nearest primal node.
//   particles per species, two structure-of-arrays buffers (ping-pong).  Each
//            tile owns a segment [seg_start[t], seg_start[t] + cap[t]) in both
//            buffers; count[t] particles of the segment are live.
//            FP64 form:  x, y, z, px, py, pz, w          (double)
//            mixed form: key (packed node index), dx, dy, dz (in-cell offset
//                        in [-0.5, 0.5), cell units), px, py, pz, w (float)
//
// One step (all on the simulation's stream, optionally one CUDA graph):
//   J <- 0; per species: k_step_particles (one CTA per tile: stage the tile's
//   E and B_m in shared memory, gather, push, Esirkepov deposit into a
//   shared J tile, write each particle to its destination tile's segment in the
//   other buffer, flush the J tile with global atomics); fold the periodic J
//   (mixed form, per-cell mode: the tile's particles are first ranked by cell and
//   loaded into shared memory in cell order, so the lanes of a warp gather from
//   the same few cells; after the push, particles that keep their node are
//   deposited per cell from register sums, the others one per thread)
//   ghosts; Ampere on all points; Faraday on all points (periodic images for the
//   boundary layer) fused with B_m <- (B_new + B_old)/2.
// A tile whose segment fills up spills particles to an overflow list; the host
// sees the spill after the step and re-lays the segments out (rare).

#include "common.cuh"
#include "resident_rad.cuh"
#include "scan.cuh"

#include <cuda.h> // CUtensorMap (the encoder is looked up through the runtime: no libcuda link)
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace sg {
namespace {

constexpr int OS = 2; // ghost width (oversize) of order-2 interpolation

struct GridInfo {
    int ndim;
    int N[3];   // cells per dimension
    int np[3];  // primal extents with ghosts (N + 1 + 2*OS); 1 for an absent dimension
    int T[3];   // tile size in cells
    int tshift[3]; // log2(T) when T is a power of two, else -1
    int nt[3];  // tiles per dimension
    int ntiles;
    int open[3]; // 1: open axis (Silver-Mueller fields, particles removed at x < 0 or x >= L)
    double dx[3], dxi[3], L[3], dt;
};

// Extent of a component with staggering flags s[] (dual adds one point).
__host__ __device__ inline int ext( const GridInfo &g, int d, int dual ) { return d < g.ndim ? g.np[d] + dual : 1; }

// Staggering of E, B, J components: comp 0..2 E/J, 3..5 B.
__host__ __device__ inline int stag( int comp, int d )
{
    // Ex(d,p,p) Ey(p,d,p) Ez(p,p,d) Bx(p,d,d) By(d,p,d) Bz(d,d,p)
    if( comp < 3 ) return d == comp ? 1 : 0;
    return d == comp - 3 ? 0 : 1;
}

// J is FP64 in both forms: the mixed form's per-tile FP32 currents are added into FP64
// global arrays, so the sum over tiles and its storage add no FP32 rounding (each
// rounding there breaks discrete charge conservation by the rounded amount).
template <class T>
struct Fields {
    T *E[3], *B[3], *Bm[3];
    double *J[3];
    T *Ec[3]; // compensation of E's FP32 sums (mixed form), else null
};

template <bool MIXED>
struct PBuf;
template <>
struct PBuf<false> {
    double *x[3];
    double *p[3];
    double *w;
    double *tau; // optical depth of a radiating species, else null
};
template <>
struct PBuf<true> {
    unsigned *key;
    float *d[3];
    float *p[3];
    float *w;
    float *tau; // optical depth of a radiating species, else null
};

struct SpecParams {
    double qm_dts2;  // charge / mass * dt / 2
    double charge;
    double mass;
    double cw;       // charge * inverse cell volume (per unit weight)
    double cr[3];    // cw * dx_d / dt: Esirkepov current factor per unit weight
    double vs[3];    // dt / dx_d: displacement in cells per unit velocity
    float f_qm_dts2, f_cw, f_cr[3], f_vs[3]; // the same in FP32 (the mixed form's kernel reads these)
    int tile0;       // first tile of the launch (block b steps tile tile0 + b)
    int *queue;        // persistent launch: counter of the next item (null: one CTA per tile)
    const int *order;  // tile of each item, relative to tile0 (null: item itself)
    int nitems;        // items of a persistent launch
};

// Packed node index of the mixed form: 3D x:11 y:10 z:10 bits, 2D x:16 y:16 bits.
__host__ __device__ inline unsigned pack_key( int ndim, int ix, int iy, int iz )
{
    return ndim == 3 ? ( ( unsigned )ix << 20 ) | ( ( unsigned )iy << 10 ) | ( unsigned )iz
                     : ( ( unsigned )ix << 16 ) | ( unsigned )iy;
}
__host__ __device__ inline void unpack_key( int ndim, unsigned k, int &ix, int &iy, int &iz )
{
    if( ndim == 3 ) {
        ix = ( int )( k >> 20 );
        iy = ( int )( ( k >> 10 ) & 1023u );
        iz = ( int )( k & 1023u );
    } else {
        ix = ( int )( k >> 16 );
        iy = ( int )( k & 65535u );
        iz = 0;
    }
}

__host__ __device__ inline int tile_div( const GridInfo &g, int i, int d )
{
    return g.tshift[d] >= 0 ? i >> g.tshift[d] : i / g.T[d];
}

__host__ __device__ inline int tile_of( const GridInfo &g, int ix, int iy, int iz )
{
    int t = tile_div( g, ix, 0 );
    t = t * g.nt[1] + tile_div( g, iy, 1 );
    if( g.ndim == 3 ) t = t * g.nt[2] + tile_div( g, iz, 2 );
    return t;
}

// Thread map for tile copies: lanes along the last dimension.  3D tiles with a
// cross section of at most 8 x 8 use 8 lanes per row and 8 rows per x plane
// (no divisions); 2D tiles with at most 16 points per row use 16 lanes per row.
// Other shapes fall back to a division per point.
// Asynchronous global -> shared copy of one 4- or 8-byte word (cp.async, sm_80+).
// When `valid` is false nothing is read (src-size 0) and the word is zero-filled;
// `src` must still be a valid address then.
template <class T>
__device__ __forceinline__ void cp_async_word( T *dst, const T *src, bool valid )
{
    static_assert( sizeof( T ) == 4 || sizeof( T ) == 8, "4- or 8-byte words" );
    const unsigned d = ( unsigned )__cvta_generic_to_shared( dst );
    const int n = valid ? ( int )sizeof( T ) : 0;
    if( sizeof( T ) == 4 )
        asm volatile( "cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"( d ), "l"( src ), "r"( n ) : "memory" );
    else
        asm volatile( "cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"( d ), "l"( src ), "r"( n ) : "memory" );
}

__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile( "cp.async.wait_all;\n" ::: "memory" );
}

struct TileMap {
    int cx0, cy, cz, step; // first x, this thread's (y, z), x stride
    bool fast, active;
};

template <int DIM>
__device__ __forceinline__ TileMap tile_map( int NY, int NZ )
{
    TileMap m;
    if( DIM == 3 && NY <= 8 && NZ <= 8 ) {
        m.cz = threadIdx.x & 7;
        m.cy = ( threadIdx.x >> 3 ) & 7;
        m.cx0 = threadIdx.x >> 6;
        m.step = blockDim.x >> 6;
        m.fast = true;
        m.active = m.cz < NZ && m.cy < NY;
    } else if( DIM == 2 && NY <= 16 ) {
        m.cz = 0;
        m.cy = threadIdx.x & 15;
        m.cx0 = threadIdx.x >> 4;
        m.step = blockDim.x >> 4;
        m.fast = true;
        m.active = m.cy < NY;
    } else {
        m.cz = m.cy = m.cx0 = m.step = 0;
        m.fast = false;
        m.active = true;
    }
    return m;
}

// ------------------------------------------------------------------------------
// The fused particle kernel.
// ------------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ T rsqrt_t( T x );
template <>
__device__ __forceinline__ double rsqrt_t<double>( double x ) { return 1.0 / sqrt( x ); }
// FP32 (mixed form): the hardware approximations (a few ulp), well inside the form's
// 1e-5 parity bar, instead of the IEEE-rounded sequences
template <>
__device__ __forceinline__ float rsqrt_t<float>( float x ) { return rsqrtf( x ); }

template <class T>
__device__ __forceinline__ T rcp_t( T x );
template <>
__device__ __forceinline__ double rcp_t<double>( double x ) { return 1.0 / x; }
template <>
__device__ __forceinline__ float rcp_t<float>( float x ) { return __fdividef( 1.0f, x ); }

template <int KIND, class T>
__device__ __forceinline__ T push_t( T qm, T Ex, T Ey, T Ez, T Bx, T By, T Bz, T &px, T &py, T &pz )
{
    if( KIND == 0 ) {
        T pxsm = qm * Ex, pysm = qm * Ey, pzsm = qm * Ez;
        const T umx = px + pxsm, umy = py + pysm, umz = pz + pzsm;
        const T lg = qm * rsqrt_t<T>( T( 1 ) + umx * umx + umy * umy + umz * umz );
        const T Tx = lg * Bx, Ty = lg * By, Tz = lg * Bz;
        const T inv_det = rcp_t<T>( T( 1 ) + Tx * Tx + Ty * Ty + Tz * Tz );
        pxsm += ( ( T( 1 ) + Tx * Tx - Ty * Ty - Tz * Tz ) * umx + T( 2 ) * ( Tx * Ty + Tz ) * umy + T( 2 ) * ( Tz * Tx - Ty ) * umz ) * inv_det;
        pysm += ( T( 2 ) * ( Tx * Ty - Tz ) * umx + ( T( 1 ) - Tx * Tx + Ty * Ty - Tz * Tz ) * umy + T( 2 ) * ( Ty * Tz + Tx ) * umz ) * inv_det;
        pzsm += ( T( 2 ) * ( Tz * Tx + Ty ) * umx + T( 2 ) * ( Ty * Tz - Tx ) * umy + ( T( 1 ) - Tx * Tx - Ty * Ty + Tz * Tz ) * umz ) * inv_det;
        px = pxsm; py = pysm; pz = pzsm;
    } else if( KIND == 1 ) {
        const T g0 = rsqrt_t<T>( T( 1 ) + px * px + py * py + pz * pz );
        T upx = px + T( 2 ) * qm * Ex, upy = py + T( 2 ) * qm * Ey, upz = pz + T( 2 ) * qm * Ez;
        T Tx = qm * Bx, Ty = qm * By, Tz = qm * Bz;
        upx += g0 * ( py * Tz - pz * Ty );
        upy += g0 * ( pz * Tx - px * Tz );
        upz += g0 * ( px * Ty - py * Tx );
        T alpha = T( 1 ) + upx * upx + upy * upy + upz * upz;
        const T T2 = Tx * Tx + Ty * Ty + Tz * Tz;
        T s = alpha - T2;
        T us2 = upx * Tx + upy * Ty + upz * Tz;
        us2 = us2 * us2;
        alpha = rsqrt_t<T>( T( 0.5 ) * ( s + sqrt( s * s + T( 4 ) * ( T2 + us2 ) ) ) );
        Tx *= alpha; Ty *= alpha; Tz *= alpha;
        s = rcp_t<T>( T( 1 ) + Tx * Tx + Ty * Ty + Tz * Tz );
        alpha = upx * Tx + upy * Ty + upz * Tz;
        px = s * ( upx + alpha * Tx + Tz * upy - Ty * upz );
        py = s * ( upy + alpha * Ty + Tx * upz - Tz * upx );
        pz = s * ( upz + alpha * Tz + Ty * upx - Tx * upy );
    } else {
        T pxsm = qm * Ex, pysm = qm * Ey, pzsm = qm * Ez;
        const T umx = px + pxsm, umy = py + pysm, umz = pz + pzsm;
        const T gfm2 = T( 1 ) + umx * umx + umy * umy + umz * umz;
        T Tx = qm * Bx, Ty = qm * By, Tz = qm * Bz;
        const T beta2 = Tx * Tx + Ty * Ty + Tz * Tz;
        const T Tum = Tx * umx + Ty * umy + Tz * umz;
        const T lg = rsqrt_t<T>( T( 0.5 ) * ( gfm2 - beta2 + sqrt( ( gfm2 - beta2 ) * ( gfm2 - beta2 ) + T( 4 ) * ( beta2 + Tum * Tum ) ) ) );
        Tx *= lg; Ty *= lg; Tz *= lg;
        const T Tx2 = Tx * Tx, Ty2 = Ty * Ty, Tz2 = Tz * Tz;
        const T TxTy = Tx * Ty, TyTz = Ty * Tz, TzTx = Tz * Tx;
        const T inv_det = rcp_t<T>( T( 1 ) + Tx2 + Ty2 + Tz2 );
        const T upx = ( ( T( 1 ) + Tx2 - Ty2 - Tz2 ) * umx + T( 2 ) * ( TxTy + Tz ) * umy + T( 2 ) * ( TzTx - Ty ) * umz ) * inv_det;
        const T upy = ( T( 2 ) * ( TxTy - Tz ) * umx + ( T( 1 ) - Tx2 + Ty2 - Tz2 ) * umy + T( 2 ) * ( TyTz + Tx ) * umz ) * inv_det;
        const T upz = ( T( 2 ) * ( TzTx + Ty ) * umx + T( 2 ) * ( TyTz - Tx ) * umy + ( T( 1 ) - Tx2 - Ty2 + Tz2 ) * umz ) * inv_det;
        px = pxsm + upx; py = pysm + upy; pz = pzsm + upz;
    }
    return rsqrt_t<T>( T( 1 ) + px * px + py * py + pz * pz );
}

struct TileDims {
    int FX, FY, FZ; // field tile extents (T + 3)
    int JX, JY, JZ; // current tile extents (T + 4)
    int JXS;        // current tile x stride: JY JZ, in 3D plus 4 words (below)
};

__host__ __device__ inline TileDims tile_dims( const GridInfo &g )
{
    TileDims t;
    t.FX = g.T[0] + 3;
    t.FY = g.T[1] + 3;
    t.FZ = g.ndim == 3 ? g.T[2] + 3 : 1;
    t.JX = g.T[0] + 4;
    t.JY = g.T[1] + 4;
    t.JZ = g.ndim == 3 ? g.T[2] + 4 : 1;
    // 3D: an x stride of 4 (mod 32) words puts the 4 x 4 x 4 cells of a 4^3 tile on the
    // 32 banks two by two (4 cx + 8 cy + cz), where JY JZ = 64 put them four by four
    // (8 cy + cz): the deposit's lanes, one per particle or per cell, conflict less
    t.JXS = t.JY * t.JZ + ( g.ndim == 3 ? 4 : 0 );
    return t;
}

// Words of one current component tile (the last x plane is not padded).
__host__ __device__ inline int jtile_size( const TileDims &t ) { return ( t.JX - 1 ) * t.JXS + t.JY * t.JZ; }
constexpr int jtile3_size( int t ) { return ( t + 3 ) * ( ( t + 4 ) * ( t + 4 ) + 4 ) + ( t + 4 ) * ( t + 4 ); }

// Gather one component from the shared tile: sum_a cx[a] sum_b cy[b] sum_c cz[c] F.
template <int DIM, class T>
__device__ __forceinline__ T gather_tile( const T *__restrict__ F, const TileDims &td, const T *cx, const T *cy,
                                          const T *cz, int bx, int by, int bz )
{
    T r = T( 0 );
#pragma unroll
    for( int a = 0; a < 3; a++ ) {
        T ra = T( 0 );
#pragma unroll
        for( int b = 0; b < 3; b++ ) {
            const T *row = F + ( ( bx + a ) * td.FY + ( by + b ) ) * td.FZ + bz;
            if( DIM == 3 ) {
                const T rb = cz[0] * row[0] + cz[1] * row[1] + cz[2] * row[2];
                ra += cy[b] * rb;
            } else {
                ra += cy[b] * row[0];
            }
        }
        r += cx[a] * ra;
    }
    return r;
}

// Two components gathered at once with paired FP32 arithmetic (FFMA2: one instruction,
// two independent IEEE fmas): the same operations as two gather_tile calls, half the
// FMA instructions.  Each component has its own weights and tile origin.
template <int DIM>
__device__ __forceinline__ float2 gather_pair( const float *__restrict__ F1, const float *__restrict__ F2,
                                               const TileDims &td, const float *cx1, const float *cx2,
                                               const float *cy1, const float *cy2, const float *cz1,
                                               const float *cz2, int bx1, int by1, int bz1, int bx2, int by2,
                                               int bz2 )
{
    float2 r = make_float2( 0.f, 0.f );
#pragma unroll
    for( int a = 0; a < 3; a++ ) {
        float2 ra = make_float2( 0.f, 0.f );
#pragma unroll
        for( int b = 0; b < 3; b++ ) {
            const float *row1 = F1 + ( ( bx1 + a ) * td.FY + ( by1 + b ) ) * td.FZ + bz1;
            const float *row2 = F2 + ( ( bx2 + a ) * td.FY + ( by2 + b ) ) * td.FZ + bz2;
            float2 rb;
            if( DIM == 3 ) {
                rb = __fmul2_rn( make_float2( cz1[0], cz2[0] ), make_float2( row1[0], row2[0] ) );
                rb = __ffma2_rn( make_float2( cz1[1], cz2[1] ), make_float2( row1[1], row2[1] ), rb );
                rb = __ffma2_rn( make_float2( cz1[2], cz2[2] ), make_float2( row1[2], row2[2] ), rb );
            } else {
                rb = make_float2( row1[0], row2[0] );
            }
            ra = __ffma2_rn( make_float2( cy1[b], cy2[b] ), rb, ra );
        }
        r = __ffma2_rn( make_float2( cx1[a], cx2[a] ), ra, r );
    }
    return r;
}

// FP32 to FP64 with integer operations (exact, every class of value): this GPU runs
// FP64 adds, compares and conversions on its FP64 pipe at 1/64 of the FP32 rate.
__device__ __forceinline__ double widen( float x )
{
    const unsigned u = __float_as_uint( x ), sgn = u & 0x80000000u, ex = ( u >> 23 ) & 0xffu, man = u & 0x7fffffu;
    unsigned e64, frac; // FP64 exponent field, 23-bit fraction
    if( ex - 1u < 254u ) {
        e64 = ex + 896u; // normal: 1023 - 127
        frac = man;
    } else if( ex == 0xffu ) {
        e64 = 0x7ffu; // infinity, NaN
        frac = man;
    } else if( man == 0u ) {
        e64 = 0u; // zero
        frac = 0u;
    } else {
        // subnormal: man 2^-149 = 1.f 2^(p - 149), p = the leading bit of man
        const int p = 31 - __clz( man );
        e64 = ( unsigned )( p + 874 );
        frac = ( man << ( 23 - p ) ) & 0x7fffffu;
    }
    return __hiloint2double( ( int )( sgn | ( e64 << 20 ) | ( frac >> 3 ) ), ( int )( frac << 29 ) );
}

// A current-tile value: the per-cell mode's two FP32 tiles (cell sums, node-changing
// particles) summed in FP32, one rounding.  to_global widens it for the FP64 arrays
// (the zero test stays in the tile's type: an FP64 compare also takes the FP64 pipe).
template <bool CELLS, class T>
__device__ __forceinline__ T tile_value( const T *a, const T *b, int e )
{
    if constexpr( CELLS ) return a[e] + b[e];
    else return a[e];
}
__device__ __forceinline__ double to_global( float v ) { return widen( v ); }
__device__ __forceinline__ double to_global( double v ) { return v; }

template <class T>
__device__ __forceinline__ void sh_add( T *a, T v )
{
    if( v != T( 0 ) ) atomicAdd( a, v );
}

// Per-dimension Esirkepov window: 4 nodes starting at lo (0 or 1) of the
// 5-point stencil; A = (S0+S1)/2, D = S1-S0, P = running sums of D.  S0 sits
// at stencil points 1..3, S1 at shift+1..shift+3; everything stays in registers
// (selects instead of indexed stores).
template <class T>
struct EsirWin {
    int lo;
    T A[4], D[4], P[3];
};

template <class T>
__device__ __forceinline__ T pick3( int j, T c0, T c1, T c2 )
{
    return j == 0 ? c0 : ( j == 1 ? c1 : ( j == 2 ? c2 : T( 0 ) ) );
}

// Deposit weights of the mixed form: the outer two on the 2^-24 grid, the middle one
// 1 minus them.  They then sum to 1 exactly, S1 - S0 and its running sums are exact in
// FP32, and the running sum over a whole window is exactly zero: the deposit breaks
// charge conservation only by the rounding of the transverse weights and products.
// (Plain FP32 weights sum to 1 only to a few ulp, a per-step error of that size at
// the window's last node.)  The FP64 form keeps the reference's weights.
template <class T>
__device__ __forceinline__ void dep_spline( T d, T &c0, T &c1, T &c2 )
{
    bspline2( d, c0, c1, c2 );
    if constexpr( sizeof( T ) == 4 ) {
        // c0, c2 lie in [0, 1/2]: adding 1/2 rounds them to the 2^-24 grid (to nearest,
        // ties to even, as rint(c 2^24) 2^-24) with one FP32 add
        c0 = __fsub_rn( __fadd_rn( c0, 0.5f ), 0.5f );
        c2 = __fsub_rn( __fadd_rn( c2, 0.5f ), 0.5f );
        c1 = ( 1.0f - c0 ) - c2;
    }
}

template <class T>
__device__ __forceinline__ void esir_win( T c0o, T c1o, T c2o, T dnew, int shift, EsirWin<T> &w )
{
    T c0, c1, c2;
    dep_spline( dnew, c0, c1, c2 );
    w.lo = shift < 0 ? 0 : 1;
    T run = T( 0 );
#pragma unroll
    for( int i = 0; i < 4; i++ ) {
        const int k = w.lo + i;
        const T s0 = pick3( k - 1, c0o, c1o, c2o );
        const T s1 = pick3( k - 1 - shift, c0, c1, c2 );
        w.A[i] = T( 0.5 ) * ( s0 + s1 );
        w.D[i] = s1 - s0;
        if( i < 3 ) {
            run += w.D[i];
            w.P[i] = run;
        }
    }
    // with no node change the sum over the whole window is S1 - S0 summed, zero up to
    // rounding: the last current node gets nothing
    if( shift == 0 ) w.P[2] = T( 0 );
}

// Esirkepov deposit of one particle straight into the shared J tile (atomics):
// Jx(d,p,p) at node (lo+1+m, lo+u, lo+v) of the 5-point stencil gets
// -cr_x P_x[m] (A_y[u] A_z[v] + D_y[u] D_z[v] / 12), and cyclically for Jy, Jz;
// in 2D, Jz = crz (A_x A_y + D_x D_y / 12) with crz = q w v_z / V.  lx = the old
// node, tile-local; the J tile origin is two nodes below the tile.
template <int DIM, class T>
__device__ __forceinline__ void deposit_direct( T *sJ, const TileDims &td, int jsz, const int *lx,
                                                const EsirWin<T> *W, const T *cr, T crz, unsigned cmask = 7u )
{
    const T twelfth = T( 1.0 / 12.0 );
    if( DIM == 3 ) {
        // one component per pass of a loop that is not unrolled (a small body: this code
        // runs once per tile); after each pass the dimensions rotate, (a, b, e) ->
        // (b, e, a), so the current's dimension a is always Wa
        EsirWin<T> Wa = W[0], Wb = W[1], We = W[2];
        int la = lx[0], lb = lx[1], le = lx[2];
        int sa = td.JXS, sb = td.JZ, se = 1;
        T ca = cr[0], cb = cr[1], ce = cr[2];
        T *J = sJ;
#pragma unroll 1
        for( int c = 0; c < 3; c++ ) {
            if( ( cmask >> c ) & 1u ) {
#pragma unroll
                for( int u = 0; u < 4; u++ )
#pragma unroll
                    for( int v = 0; v < 4; v++ ) {
                        const T wgt = Wb.A[u] * We.A[v] + twelfth * Wb.D[u] * We.D[v];
                        const int base = ( la + Wa.lo + 1 ) * sa + ( lb + Wb.lo + u ) * sb + ( le + We.lo + v ) * se;
#pragma unroll
                        for( int m = 0; m < 3; m++ ) sh_add( &J[base + m * sa], -ca * Wa.P[m] * wgt );
                    }
            }
            const EsirWin<T> tw = Wa;
            Wa = Wb; Wb = We; We = tw;
            int ti = la;
            la = lb; lb = le; le = ti;
            ti = sa;
            sa = sb; sb = se; se = ti;
            const T tc = ca;
            ca = cb; cb = ce; ce = tc;
            J += jsz;
        }
    } else {
        T *J0 = sJ, *J1 = sJ + jsz, *J2 = sJ + 2 * jsz;
        if( cmask & 1u ) {
#pragma unroll
            for( int u = 0; u < 4; u++ ) {
                const T ay = W[1].A[u];
#pragma unroll
                for( int m = 0; m < 3; m++ )
                    sh_add( &J0[( lx[0] + W[0].lo + 1 + m ) * td.JXS + lx[1] + W[1].lo + u], -cr[0] * W[0].P[m] * ay );
            }
        }
        if( cmask & 2u ) {
#pragma unroll
            for( int u = 0; u < 4; u++ ) {
                const T ax = W[0].A[u];
#pragma unroll
                for( int m = 0; m < 3; m++ )
                    sh_add( &J1[( lx[0] + W[0].lo + u ) * td.JXS + lx[1] + W[1].lo + 1 + m], -cr[1] * W[1].P[m] * ax );
            }
        }
        if( cmask & 4u ) {
#pragma unroll
            for( int u = 0; u < 4; u++ )
#pragma unroll
                for( int v = 0; v < 4; v++ ) {
                    const T wz = W[0].A[u] * W[1].A[v] + twelfth * W[0].D[u] * W[1].D[v];
                    sh_add( &J2[( lx[0] + W[0].lo + u ) * td.JXS + lx[1] + W[1].lo + v], crz * wz );
                }
        }
    }
}

// Footprint weights of one dimension for the per-cell deposit: S0 (old weights o) and
// S1 (new weights n, on the new node) on the old node's stencil points 1..3.  A shift
// s = +-1 moves S1 by s; the weight it moves out of the footprint (to point 4 for s = 1,
// 0 for s = -1) is returned in nov.  A = (S0 + S1) / 2, D = S1 - S0, P = the running
// sums of S1 - S0 up to points 1 and 2 (the current at points 2 and 3; point 0 holds
// nov when s = -1).
template <class T>
__device__ __forceinline__ void footprint_weights( T dold, T dnew, int s, T *A, T *D, T *P, T &nov )
{
    T o0, o1, o2, n0, n1, n2;
    dep_spline( dold, o0, o1, o2 );
    dep_spline( dnew, n0, n1, n2 );
    const T f0 = s > 0 ? T( 0 ) : ( s < 0 ? n1 : n0 );
    const T f1 = s > 0 ? n0 : ( s < 0 ? n2 : n1 );
    const T f2 = s > 0 ? n1 : ( s < 0 ? T( 0 ) : n2 );
    nov = s > 0 ? n2 : n0;
    A[0] = T( 0.5 ) * ( o0 + f0 ); A[1] = T( 0.5 ) * ( o1 + f1 ); A[2] = T( 0.5 ) * ( o2 + f2 );
    D[0] = f0 - o0; D[1] = f1 - o1; D[2] = f2 - o2;
    P[0] = D[0] + ( s < 0 ? nov : T( 0 ) );
    P[1] = P[0] + D[1];
}

// footprint_weights for dimensions 0 and 1 at once in paired FP32 arithmetic (FADD2,
// FMUL2: two IEEE operations per instruction), then dimension 2: the same formulas,
// the splines rounded to the 2^-24 grid as dep_spline rounds them.
__device__ __forceinline__ float2 neg2( float2 a ) { return make_float2( -a.x, -a.y ); }

__device__ __forceinline__ void dep_spline2( float2 d, float2 &c0, float2 &c1, float2 &c2 )
{
    const float2 half = make_float2( 0.5f, 0.5f ), quarter = make_float2( 0.25f, 0.25f );
    const float2 d2 = __fmul2_rn( d, d );
    c0 = __fmul2_rn( half, __fadd2_rn( __fadd2_rn( d2, neg2( d ) ), quarter ) );
    c2 = __fmul2_rn( half, __fadd2_rn( __fadd2_rn( d2, d ), quarter ) );
    c0 = __fadd2_rn( __fadd2_rn( c0, half ), neg2( half ) );
    c2 = __fadd2_rn( __fadd2_rn( c2, half ), neg2( half ) );
    c1 = __fadd2_rn( __fadd2_rn( make_float2( 1.0f, 1.0f ), neg2( c0 ) ), neg2( c2 ) );
}

// Dimensions 0 and 1 of footprint_weights in paired FP32 arithmetic.
__device__ __forceinline__ void footprint_weights_xy( const float *dold, const float *dnew, const int *s,
                                                      float ( *A )[3], float ( *D )[3], float ( *P )[2], float *nov )
{
    {
        float2 o0, o1, o2, n0, n1, n2;
        dep_spline2( make_float2( dold[0], dold[1] ), o0, o1, o2 );
        dep_spline2( make_float2( dnew[0], dnew[1] ), n0, n1, n2 );
        const float2 z = make_float2( 0.f, 0.f );
        // the shift selects, lane by lane
        const float2 f0 = make_float2( s[0] > 0 ? 0.f : ( s[0] < 0 ? n1.x : n0.x ), s[1] > 0 ? 0.f : ( s[1] < 0 ? n1.y : n0.y ) );
        const float2 f1 = make_float2( s[0] > 0 ? n0.x : ( s[0] < 0 ? n2.x : n1.x ), s[1] > 0 ? n0.y : ( s[1] < 0 ? n2.y : n1.y ) );
        const float2 f2 = make_float2( s[0] > 0 ? n1.x : ( s[0] < 0 ? 0.f : n2.x ), s[1] > 0 ? n1.y : ( s[1] < 0 ? 0.f : n2.y ) );
        const float2 nv = make_float2( s[0] > 0 ? n2.x : n0.x, s[1] > 0 ? n2.y : n0.y );
        const float2 half = make_float2( 0.5f, 0.5f );
        const float2 a0 = __fmul2_rn( half, __fadd2_rn( o0, f0 ) ), a1 = __fmul2_rn( half, __fadd2_rn( o1, f1 ) ),
                     a2 = __fmul2_rn( half, __fadd2_rn( o2, f2 ) );
        const float2 e0 = __fadd2_rn( f0, neg2( o0 ) ), e1 = __fadd2_rn( f1, neg2( o1 ) ), e2 = __fadd2_rn( f2, neg2( o2 ) );
        const float2 p0 = __fadd2_rn( e0, make_float2( s[0] < 0 ? nv.x : 0.f, s[1] < 0 ? nv.y : 0.f ) );
        const float2 p1 = __fadd2_rn( p0, e1 );
        ( void )z;
        A[0][0] = a0.x; A[0][1] = a1.x; A[0][2] = a2.x;
        A[1][0] = a0.y; A[1][1] = a1.y; A[1][2] = a2.y;
        D[0][0] = e0.x; D[0][1] = e1.x; D[0][2] = e2.x;
        D[1][0] = e0.y; D[1][1] = e1.y; D[1][2] = e2.y;
        P[0][0] = p0.x; P[0][1] = p1.x;
        P[1][0] = p0.y; P[1][1] = p1.y;
        nov[0] = nv.x;
        nov[1] = nv.y;
    }
}

template <class T>
__device__ __forceinline__ void footprint_weights3( const T *dold, const T *dnew, const int *s, T ( *A )[3], T ( *D )[3],
                                                    T ( *P )[2], T *nov )
{
    if constexpr( sizeof( T ) == 4 ) {
        footprint_weights_xy( dold, dnew, s, A, D, P, nov );
        // z: its old and new splines as one pair, then footprint_weights' formulas
        float2 c0, c1, c2;
        dep_spline2( make_float2( dold[2], dnew[2] ), c0, c1, c2 );
        const int sz = s[2];
        const float o0 = c0.x, o1 = c1.x, o2 = c2.x, n0 = c0.y, n1 = c1.y, n2 = c2.y;
        const float f0 = sz > 0 ? 0.f : ( sz < 0 ? n1 : n0 );
        const float f1 = sz > 0 ? n0 : ( sz < 0 ? n2 : n1 );
        const float f2 = sz > 0 ? n1 : ( sz < 0 ? 0.f : n2 );
        nov[2] = sz > 0 ? n2 : n0;
        A[2][0] = 0.5f * ( o0 + f0 ); A[2][1] = 0.5f * ( o1 + f1 ); A[2][2] = 0.5f * ( o2 + f2 );
        D[2][0] = f0 - o0; D[2][1] = f1 - o1; D[2][2] = f2 - o2;
        P[2][0] = D[2][0] + ( sz < 0 ? nov[2] : 0.f );
        P[2][1] = P[2][0] + D[2][1];
    } else {
#pragma unroll
        for( int d = 0; d < 3; d++ ) footprint_weights<T>( dold[d], dnew[d], s[d], A[d], D[d], P[d], nov[d] );
    }
}

template <class T>
__device__ __forceinline__ T pick4( int i, T a0, T a1, T a2, T a3 )
{
    return i == 0 ? a0 : ( i == 1 ? a1 : ( i == 2 ? a2 : a3 ) );
}

// The part of a 3D Esirkepov deposit outside the old cell's footprint, for a particle
// that changes node (shift sh[d] in dimension d; the per-cell pass adds the footprint
// part).  A shifted dimension's window reaches one plane further: stencil point 4 for
// s = 1; for s = -1 point 0 across a current and point 1 along it.  In the frame of
// current component a (transverse b, e), window index 3 (across) or 2 (along) is that
// plane, with A = nov / 2, D = nov (S0 is zero there) across and Q = -s nov (the sum of
// S1 - S0 before it) along.  J_a gets -cr_a P_a (A_b A_e + D_b D_e / 12) on the points
// with at least one index beyond the footprint: 21 for a shift in one dimension.  The
// loops are not unrolled (this code runs about once per tile per warp, where fetching a
// long unrolled body costs more than running a short loop).
template <class T>
__device__ __forceinline__ void deposit_beyond( T *J2, int jsz, int jxs, int jz, const int *cl, const T ( *A )[3],
                                                const T ( *D )[3], const T ( *P )[2], const T *cr, const T *nov,
                                                const int *sh )
{
    const T twelfth = T( 1.0 / 12.0 );
#pragma unroll 1
    for( int c = 0; c < 3; c++ ) {
        const int b = c == 2 ? 0 : c + 1, e = c == 0 ? 2 : c - 1;
#define SG_SEL( x, i ) ( ( i ) == 0 ? x[0] : ( ( i ) == 1 ? x[1] : x[2] ) )
        const int sa = c == 0 ? jxs : ( c == 1 ? jz : 1 ), sb = b == 0 ? jxs : ( b == 1 ? jz : 1 ), se = e == 0 ? jxs : ( e == 1 ? jz : 1 );
        const int la = SG_SEL( cl, c ), lb = SG_SEL( cl, b ), le = SG_SEL( cl, e );
        const int s_a = SG_SEL( sh, c ), s_b = SG_SEL( sh, b ), s_e = SG_SEL( sh, e );
        const T cra = SG_SEL( cr, c ), nva = SG_SEL( nov, c ), nvb = SG_SEL( nov, b ), nve = SG_SEL( nov, e );
        T Ab[3], Db[3], Ae[3], De[3], Pa[2];
#pragma unroll
        for( int i = 0; i < 3; i++ ) {
            Ab[i] = b == 0 ? A[0][i] : ( b == 1 ? A[1][i] : A[2][i] );
            Db[i] = b == 0 ? D[0][i] : ( b == 1 ? D[1][i] : D[2][i] );
            Ae[i] = e == 0 ? A[0][i] : ( e == 1 ? A[1][i] : A[2][i] );
            De[i] = e == 0 ? D[0][i] : ( e == 1 ? D[1][i] : D[2][i] );
        }
        Pa[0] = SG_SEL( P, c )[0];
        Pa[1] = SG_SEL( P, c )[1];
#undef SG_SEL
        const T Ab3 = T( 0.5 ) * nvb, Db3 = twelfth * nvb, Ae3 = T( 0.5 ) * nve, De3 = nve;
        const T qa = s_a > 0 ? -nva : nva;
        const int pa = la + ( s_a > 0 ? 4 : 1 ), pb = lb + ( s_b > 0 ? 4 : 0 ), pe = le + ( s_e > 0 ? 4 : 0 );
        const int nu = s_b != 0 ? 4 : 3, nv = s_e != 0 ? 4 : 3;
        T *J = J2 + c * jsz;
        // the along plane beyond (index 2): every (b, e) point of the window
        if( s_a != 0 ) {
            const T ca = -( cra * qa );
#pragma unroll 1
            for( int u = 0; u < nu; u++ ) {
                const T ab = pick4( u, Ab[0], Ab[1], Ab[2], Ab3 ), db = pick4( u, twelfth * Db[0], twelfth * Db[1], twelfth * Db[2], Db3 );
                const int ib = u < 3 ? lb + 1 + u : pb;
                // (the innermost loops are unrolled: independent adds in flight together)
#pragma unroll
                for( int v = 0; v < 4; v++ ) {
                    if( v >= nv ) break;
                    const T ae = pick4( v, Ae[0], Ae[1], Ae[2], Ae3 ), de = pick4( v, De[0], De[1], De[2], De3 );
                    const int ie = v < 3 ? le + 1 + v : pe;
                    sh_add( &J[pa * sa + ib * sb + ie * se], ca * ( ab * ae + db * de ) );
                }
            }
        }
        // the across-b plane beyond (index 3) at the two footprint points along
        if( s_b != 0 ) {
#pragma unroll 1
            for( int m = 0; m < 2; m++ ) {
                const T cm = -( cra * ( m ? Pa[1] : Pa[0] ) );
#pragma unroll
                for( int v = 0; v < 4; v++ ) {
                    if( v >= nv ) break;
                    const T ae = pick4( v, Ae[0], Ae[1], Ae[2], Ae3 ), de = pick4( v, De[0], De[1], De[2], De3 );
                    const int ie = v < 3 ? le + 1 + v : pe;
                    sh_add( &J[( la + 2 + m ) * sa + pb * sb + ie * se], cm * ( Ab3 * ae + Db3 * de ) );
                }
            }
        }
        // the across-e plane beyond, footprint points of b (the corner is in the plane above)
        if( s_e != 0 ) {
#pragma unroll 1
            for( int m = 0; m < 2; m++ ) {
                const T cm = -( cra * ( m ? Pa[1] : Pa[0] ) );
#pragma unroll
                for( int u = 0; u < 3; u++ ) {
                    const T ab = u == 0 ? Ab[0] : ( u == 1 ? Ab[1] : Ab[2] ), db = u == 0 ? Db[0] : ( u == 1 ? Db[1] : Db[2] );
                    sh_add( &J[( la + 2 + m ) * sa + ( lb + 1 + u ) * sb + pe * se], cm * ( ab * Ae3 + twelfth * db * De3 ) );
                }
            }
        }
    }
}

// Per-cell mode keeps the tile's particles in shared memory in cell order, as
// REC planes of nmax words (plane k of slot s at k * nmax + s).  Loaded state:
// planes 0-2 in-cell offsets, 3-5 momenta, 7 weight.  After the push the slot
// becomes the deposit record: planes 3-5 new offsets (2D: 3-4 new offsets, 5
// v_z), plane 6 the packed node shifts; planes 0-2 and 7 are kept.
constexpr int REC = 8;
constexpr int NO_SHIFT = 1 | ( 1 << 2 ) | ( 1 << 4 ); // packed shifts (s + 1 per 2 bits) of a particle that keeps its node
constexpr int GONE_RECORD = 1 << 8;                  // record of a particle removed at an open boundary: deposits nothing

// Shared memory of the per-cell mode: REC planes of nmax floats, a count and a
// start per cell, a packed (cell, rank) word per particle (later the node-changing
// list), the list grouped by crossing dimension with each group padded to whole warps
// (nmax + LIST_PAD words; with TMA staging it uses the field tile instead), a cell
// byte per slot.
constexpr size_t CELLS_SMEM_TARGET = 44 * 1024; // five 128-thread blocks per SM
constexpr int LIST_PAD = 128;                   // four groups, each padded by at most 31
constexpr size_t cells_smem_bytes( int tc, int nmax, bool grouped )
{
    return ( size_t )REC * 4 * nmax + ( size_t )8 * tc + ( size_t )4 * nmax + ( grouped ? ( size_t )4 * ( nmax + LIST_PAD ) : 0 ) +
           ( ( ( size_t )nmax + 15 ) & ~( size_t )15 );
}

// Particles per chunk of the per-cell mode that fit CELLS_SMEM_TARGET with a tile
// of tc cells whose field and current tiles take tile_bytes (0: none fit).
constexpr int cells_chunk_fit( size_t tile_bytes, int tc, bool grouped )
{
    const size_t fixed = tile_bytes + cells_smem_bytes( tc, 0, grouped ) + 16;
    const size_t per = ( size_t )REC * 4 + ( grouped ? 8 : 4 ) + 1; // planes, rank (and grouped list) words, cell byte
    return fixed < CELLS_SMEM_TARGET ? ( int )( ( CELLS_SMEM_TARGET - fixed ) / per ) : 0;
}

// Field tile staged by the tensor memory accelerator (TMA, 3D 4x4x4 tiles): one
// cp.async.bulk.tensor per component copies a box of 8 (z) x 7 (y) x 7 (x) FP32 values.
// The box's z extent must be a multiple of 16 bytes and its start 16-byte aligned, so it
// starts at the tile's first node (4 tz) rather than one below (4 tz + 1 in array
// indices) and is 8 wide; the gather then indexes z one further.  Each component's tile
// starts on a 128-byte boundary of shared memory.  The global arrays need rows that are a
// multiple of 16 bytes, which the reference layout's 261- or 262-value rows are not: the
// step copies E and B_m into padded arrays (rows of a multiple of 4 values) first.
constexpr int TMA_BOX_Z = 8, TMA_BOX_Y = 7, TMA_BOX_X = 7;
constexpr int TMA_FSZ = 416; // floats per component tile: 8 x 7 x 7 = 392, rounded up to 128 bytes
constexpr unsigned TMA_TX_BYTES = 6 * TMA_BOX_Z * TMA_BOX_Y * TMA_BOX_X * 4;
struct TmaFields {
    CUtensorMap m[6]; // Ex Ey Ez Bx_m By_m Bz_m over the padded arrays
};

// Tile shapes with their own kernel instances (code FT): 0 any shape (runtime), 1 the
// default (4x4x4 in 3D, 8x8 in 2D), 2 8x16 (2D), 3 4x4 (2D); the 2D ones are the shapes
// the autotuner picks for the wakefield and for dense bunches.
constexpr int ft_tile( int dim, int ft, int d )
{
    return dim == 3 ? ( d < 3 ? 4 : 1 ) : ( d == 2 ? 1 : ( ft == 2 ? ( d == 0 ? 8 : 16 ) : ( ft == 3 ? 4 : 8 ) ) );
}
constexpr int ft_shift( int t ) { return t == 16 ? 4 : ( t == 8 ? 3 : ( t == 4 ? 2 : 0 ) ); }

// The chunk of such a shape: FP32 tiles of 6 field and 3 + 3 current components (the
// per-cell sums' tile and the node-changing particles' tile) with T + 3 and T + 4
// points per dimension.
constexpr int fixt_chunk( int dim, int ft )
{
    return dim == 3 ? cells_chunk_fit( ( size_t )( 6 * 7 * 7 * 7 + 6 * jtile3_size( 4 ) ) * 4, 64, true ) & ~31
                    : cells_chunk_fit( ( size_t )( 6 * ( ft_tile( 2, ft, 0 ) + 3 ) * ( ft_tile( 2, ft, 1 ) + 3 ) +
                                                   6 * ( ft_tile( 2, ft, 0 ) + 4 ) * ( ft_tile( 2, ft, 1 ) + 4 ) ) * 4,
                                       ft_tile( 2, ft, 0 ) * ft_tile( 2, ft, 1 ), true ) & ~31;
}

// The per-cell mode's second current tile (node-changing particles), FP32.
inline size_t cells_j2_bytes( const TileDims &td ) { return ( size_t )3 * jtile_size( td ) * 4; }

// The 3D default tile's chunk with TMA staging: the padded field tile (6 TMA_FSZ floats)
// and 128 bytes to align the dynamic shared memory.
constexpr size_t TMA_TILE_BYTES = ( size_t )( 6 * TMA_FSZ + 6 * jtile3_size( 4 ) ) * 4 + 128;
constexpr int tma_chunk() { return cells_chunk_fit( TMA_TILE_BYTES, 64, false ) & ~31; }

// FT > 0: the tile shape is known at compile time, so tile and stencil offsets fold into
// immediates; the chunk is fixt_chunk.
// Waits (every thread) for phase `phase` of the TMA barrier, at most a bounded number of
// polls (each try_wait itself suspends for a while); a barrier that never completes
// sets SG_ERR_STATE in the status word and returns, so the step reports the failure.
__device__ __forceinline__ void tma_wait( unsigned long long *bar, unsigned phase, int *status )
{
    const unsigned mb = ( unsigned )__cvta_generic_to_shared( bar );
    for( int it = 0; it < ( 1 << 22 ); it++ ) {
        unsigned done;
        asm volatile( "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                      : "=r"( done ) : "r"( mb ), "r"( phase ) : "memory" );
        if( done ) return;
    }
    atomicCAS( status, 0, SG_ERR_STATE );
}

// One thread arms the TMA barrier with the tile's bytes and issues the six tensor
// copies of E and B_m into sF (component c at c * fsz floats, 128-byte aligned).
__device__ __forceinline__ void tma_issue( const TmaFields &tma, unsigned long long *bar, float *sF, int fsz, int ix0,
                                           int iy0, int iz0 )
{
    const unsigned mb = ( unsigned )__cvta_generic_to_shared( bar );
    // earlier reads and writes of sF by the threads come before these asynchronous writes
    asm volatile( "fence.proxy.async.shared::cta;\n" ::: "memory" );
    asm volatile( "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"( mb ), "r"( TMA_TX_BYTES ) : "memory" );
    // box origin: z at the tile's first node (16-byte aligned), y and x one node below
    const int z0 = iz0, y0 = iy0 + OS - 1, x0 = ix0 + OS - 1;
#pragma unroll
    for( int c = 0; c < 6; c++ ) {
        const unsigned dst = ( unsigned )__cvta_generic_to_shared( sF + c * fsz );
        asm volatile( "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n"
                      ::"r"( dst ), "l"( reinterpret_cast<uint64_t>( &tma.m[c] ) ), "r"( z0 ), "r"( y0 ), "r"( x0 ), "r"( mb )
                      : "memory" );
    }
}

// TMA (3D, mixed, per-cell, FT 1 only): the field tile comes from the tensor maps in
// `tma` (padded copies of E and B_m), not from word copies.
template <int DIM, bool MIXED, int KIND, bool CELLS, int FT = 0, bool TMA = false>
__global__ void __launch_bounds__( 128, CELLS ? 5 : ( MIXED ? 8 : 4 ) ) k_step_particles(
    GridInfo g_arg, Fields<typename std::conditional<MIXED, float, double>::type> f, SpecParams sp, PBuf<MIXED> in,
    PBuf<MIXED> out, const int64_t *__restrict__ seg_start, const int *__restrict__ cap,
    const int *__restrict__ count_in, int *__restrict__ count_out, PBuf<MIXED> ovf, int *__restrict__ ovf_tile,
    int *__restrict__ ovf_count, int ovf_cap, int *__restrict__ status, int nmax_arg, int *__restrict__ removed,
    const __grid_constant__ TmaFields tma )
{
    using T = typename std::conditional<MIXED, float, double>::type;
    static_assert( !TMA || ( DIM == 3 && MIXED && CELLS && FT == 1 ), "TMA staging: 3D mixed per-cell 4x4x4 tiles" );
    const int nmax = FT ? ( TMA ? tma_chunk() : fixt_chunk( DIM, FT ) ) : nmax_arg;
    GridInfo g = g_arg;
    if constexpr( FT > 0 ) {
#pragma unroll
        for( int d = 0; d < 3; d++ ) {
            g.T[d] = ft_tile( DIM, FT, d );
            g.tshift[d] = ft_shift( ft_tile( DIM, FT, d ) );
        }
    }
    extern __shared__ __align__( 16 ) unsigned char smem_raw[];
    // TMA writes 128-byte aligned component tiles (the dynamic region is 16-byte aligned)
    T *sF = reinterpret_cast<T *>( TMA ? ( smem_raw + ( ( 128 - ( ( unsigned )__cvta_generic_to_shared( smem_raw ) & 127u ) ) & 127u ) )
                                       : smem_raw );
    TileDims td = tile_dims( g );
    if constexpr( TMA ) td.FZ = TMA_BOX_Z;
    const int fsz = TMA ? TMA_FSZ : td.FX * td.FY * td.FZ;
    const int jsz = jtile_size( td );
    T *sJ = sF + 6 * fsz;
    // per-cell mode (CELLS): particle planes, per-cell counts and starts, each
    // particle's (cell << 16 | rank in cell), each slot's cell
    const int TC = g.T[0] * g.T[1] * ( DIM == 3 ? g.T[2] : 1 );
    // per-cell mode: node-changing particles deposit into a second tile sJ2 (in 3D the
    // part of their window outside the cell's footprint).  Their single adds then round
    // against their own small partial sums, not against the per-cell sums (an FP32 add's
    // error is about an ulp of the partial sum); the flush adds the two tiles.
    T *sJ2 = sJ + 3 * jsz;
    float *sRec = reinterpret_cast<float *>( sJ2 + ( CELLS ? 3 * jsz : 0 ) );
    int *sCnt = reinterpret_cast<int *>( sRec + ( CELLS ? REC * nmax : 0 ) );
    int *sStart = sCnt + TC;
    // reused after loading as the list of node-changing slots, which the particle
    // loop's end groups by crossing dimension into sXs, each group padded to whole
    // warps (slot -1) so that a warp takes one kind only: its own array, or with TMA
    // staging the field tile, which the deposit no longer reads (a tile's next chunk
    // stages it again)
    int *sRank = sStart + TC;
    int *sXs = TMA ? reinterpret_cast<int *>( sF ) : sRank + ( CELLS ? nmax : 0 );
    unsigned char *sSlotCell = reinterpret_cast<unsigned char *>( TMA ? sRank + ( CELLS ? nmax : 0 )
                                                                      : sXs + ( CELLS ? nmax + LIST_PAD : 0 ) );
    __shared__ int sNX;         // length of that list
    __shared__ int sNT;         // length of the grouped, padded list
    __shared__ int sXc[4];      // node-changing particles per class (one dimension x, y, z; several)
    __shared__ int sXn[4];      // the same counts, kept
    __shared__ int sXb[4];      // class starts, kept

    // TMA completion barrier: thread 0 arms it per tile with the bytes to expect, the
    // copies complete it, every thread waits on its phase (bounded)
    __shared__ __align__( 8 ) unsigned long long sTmaBar;
    unsigned tma_phase = 0;
    if constexpr( TMA ) {
        if( threadIdx.x == 0 ) {
            const unsigned mb = ( unsigned )__cvta_generic_to_shared( &sTmaBar );
            asm volatile( "mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"( mb ) : "memory" );
            asm volatile( "fence.mbarrier_init.release.cluster;\n" ::: "memory" );
        }
        __syncthreads();
    }
    bool tma_pending = false;

    // One tile per CTA, or (sp.queue set) a persistent grid whose CTAs take tiles from
    // a device counter until none is left, in the order sp.order gives (densest first).
    __shared__ int sItem;
    for( int item = blockIdx.x;; ) {
    if( sp.queue ) {
        __syncthreads(); // the previous tile is done with shared memory
        if( threadIdx.x == 0 ) sItem = atomicAdd( sp.queue, 1 );
        __syncthreads();
        item = sItem;
        if( item >= sp.nitems ) break;
    }
    const int tile = sp.tile0 + ( sp.order ? sp.order[item] : item );
    int tz = 0, ty, tx;
    if( DIM == 3 ) {
        tz = tile % g.nt[2];
        ty = ( tile / g.nt[2] ) % g.nt[1];
        tx = tile / ( g.nt[2] * g.nt[1] );
    } else {
        ty = tile % g.nt[1];
        tx = tile / g.nt[1];
    }
    const int ix0 = tx * g.T[0], iy0 = ty * g.T[1], iz0 = DIM == 3 ? tz * g.T[2] : 0;

    // 1. stage E and B_m (field tile origin = array index (i0 + OS - 1)) and clear J
    if constexpr( TMA ) {
        if( threadIdx.x == 0 ) tma_issue( tma, &sTmaBar, sF, fsz, ix0, iy0, iz0 );
        tma_pending = true;
    }
    const TileMap fm = tile_map<DIM>( td.FY, td.FZ );
#pragma unroll
    for( int c = 0; c < ( TMA ? 0 : 6 ); c++ ) {
        const T *src = c < 3 ? f.E[c] : f.Bm[c - 3];
        const int ny = ext( g, 1, stag( c, 1 ) ), nz = ext( g, 2, stag( c, 2 ) );
        const int nx = ext( g, 0, stag( c, 0 ) );
        T *dst = sF + c * fsz;
        // asynchronous copies: every word of the tile is in flight at once
        if( fm.fast ) {
            if( fm.active ) {
                const int gy = iy0 + OS - 1 + fm.cy, gz = DIM == 3 ? iz0 + OS - 1 + fm.cz : 0;
                for( int cx = fm.cx0; cx < td.FX; cx += fm.step ) {
                    const int gx = ix0 + OS - 1 + cx;
                    const bool in = gx < nx && gy < ny && gz < nz;
                    cp_async_word( &dst[( cx * td.FY + fm.cy ) * td.FZ + fm.cz],
                                   in ? &src[( ( int64_t )gx * ny + gy ) * nz + gz] : src, in );
                }
            }
        } else {
            for( int e = threadIdx.x; e < fsz; e += blockDim.x ) {
                const int cz = e % td.FZ, cy = ( e / td.FZ ) % td.FY, cx = e / ( td.FZ * td.FY );
                const int gx = ix0 + OS - 1 + cx, gy = iy0 + OS - 1 + cy, gz = DIM == 3 ? iz0 + OS - 1 + cz : 0;
                const bool in = gx < nx && gy < ny && gz < nz;
                cp_async_word( &dst[e], in ? &src[( ( int64_t )gx * ny + gy ) * nz + gz] : src, in );
            }
        }
    }
    for( int e = threadIdx.x; e < ( CELLS ? 6 : 3 ) * jsz; e += blockDim.x ) sJ[e] = T( 0 );
    // per-cell mode keeps the field copies in flight through the ranking and waits
    // for them together with the particle copies
    if constexpr( !CELLS ) cp_async_wait_all();
    __syncthreads();

    // (FP32 copies for the mixed form: a conversion from FP64 takes the FP64 pipe)
    const T qm = MIXED ? T( sp.f_qm_dts2 ) : T( sp.qm_dts2 );
    const T vs[3] = { MIXED ? T( sp.f_vs[0] ) : T( sp.vs[0] ), MIXED ? T( sp.f_vs[1] ) : T( sp.vs[1] ),
                      MIXED ? T( sp.f_vs[2] ) : T( sp.vs[2] ) };
    const T cr3[3] = { MIXED ? T( sp.f_cr[0] ) : T( sp.cr[0] ), MIXED ? T( sp.f_cr[1] ) : T( sp.cr[1] ),
                       MIXED ? T( sp.f_cr[2] ) : T( sp.cr[2] ) };
    const T cw0 = MIXED ? T( sp.f_cw ) : T( sp.cw );
    const unsigned lane = threadIdx.x & 31u;

    // Per-cell mode takes the tile's particles in chunks of at most nmax (the
    // shared planes' capacity), so a dense tile costs more passes, not more
    // shared memory; the J tile accumulates over the chunks.  The FP64 form
    // makes one pass over the whole tile.
    const int ntot = count_in[tile];
    const int64_t seg0 = seg_start[tile];
    for( int c0 = 0; c0 < ( CELLS ? ntot : 1 ); c0 += ( CELLS ? nmax : 1 ) ) {
    const int n = CELLS ? min( nmax, ntot - c0 ) : ntot;
    const int64_t s0 = seg0 + c0;
    if constexpr( TMA ) {
        // the previous chunk kept its node-changing list in the field tile: stage it again
        if( c0 > 0 ) {
            if( threadIdx.x == 0 ) tma_issue( tma, &sTmaBar, sF, fsz, ix0, iy0, iz0 );
            tma_pending = true;
        }
    }
    if constexpr( CELLS ) {
        // rank of every particle inside its cell, then the cells' start offsets
        for( int c = threadIdx.x; c < TC; c += blockDim.x ) sCnt[c] = 0;
        __syncthreads();
        constexpr int KB = 4; // keys loaded per thread before ranking (independent loads in flight)
        for( int qb = threadIdx.x; qb < n; qb += KB * blockDim.x ) {
            unsigned key[KB];
#pragma unroll
            for( int j = 0; j < KB; j++ ) {
                const int q = qb + j * blockDim.x;
                key[j] = q < n ? in.key[s0 + q] : 0u;
            }
#pragma unroll
            for( int j = 0; j < KB; j++ ) {
                const int q = qb + j * blockDim.x;
                if( q >= n ) break;
                int gx, gy, gz;
                unpack_key( DIM, key[j], gx, gy, gz );
                int l0 = gx - ix0, l1 = gy - iy0, l2 = DIM == 3 ? gz - iz0 : 0;
                if( l0 < 0 || l0 >= g.T[0] || l1 < 0 || l1 >= g.T[1] || ( DIM == 3 && ( l2 < 0 || l2 >= g.T[2] ) ) ) {
                    atomicCAS( status, 0, SG_ERR_BOUNDS );
                    l0 = l1 = l2 = 0;
                }
                const int lc = DIM == 3 ? ( l0 * g.T[1] + l1 ) * g.T[2] + l2 : l0 * g.T[1] + l1;
                sRank[q] = ( lc << 16 ) | atomicAdd( &sCnt[lc], 1 );
            }
        }
        __syncthreads();
        if( threadIdx.x < 32 ) {
            int run = 0;
            for( int base = 0; base < TC; base += 32 ) {
                const int c = base + ( int )threadIdx.x;
                const int v = c < TC ? sCnt[c] : 0;
                int x = v;
#pragma unroll
                for( int o = 1; o < 32; o <<= 1 ) {
                    const int y = __shfl_up_sync( 0xffffffffu, x, o );
                    if( ( int )threadIdx.x >= o ) x += y;
                }
                if( c < TC ) sStart[c] = run + x - v;
                run += __shfl_sync( 0xffffffffu, x, 31 );
            }
        }
        __syncthreads();
        // load the tile's particles into their cell-ordered slots (coalesced reads)
        for( int q = threadIdx.x; q < n; q += blockDim.x ) {
            const int v = sRank[q];
            const int lc = v >> 16;
            const int slot = sStart[lc] + ( v & 0xffff );
            const int64_t src = s0 + q;
#pragma unroll
            for( int d = 0; d < DIM; d++ ) cp_async_word( &sRec[d * nmax + slot], &in.d[d][src], true );
#pragma unroll
            for( int k = 0; k < 3; k++ ) cp_async_word( &sRec[( 3 + k ) * nmax + slot], &in.p[k][src], true );
            cp_async_word( &sRec[7 * nmax + slot], &in.w[src], true );
            // a radiating species' optical depth rides in the record plane until the record is written
            if( in.tau ) cp_async_word( &sRec[6 * nmax + slot], &in.tau[src], true );
            sSlotCell[slot] = ( unsigned char )lc;
        }
        if( threadIdx.x == 0 ) {
            sNX = 0;
        }
        if( threadIdx.x < 4 ) sXc[threadIdx.x] = 0;
        cp_async_wait_all(); // the particle planes (and, on the first chunk, the field tile)
        if constexpr( TMA ) {
            if( tma_pending ) {
                tma_wait( &sTmaBar, tma_phase, status );
                tma_phase ^= 1u;
                tma_pending = false;
            }
        }
        __syncthreads();
    }

    for( int base = 0; base < n; base += blockDim.x ) {
        const int q = base + threadIdx.x;
        const bool valid = q < n;
        const int64_t src = s0 + ( valid ? q : 0 );
        // ---- load the particle ------------------------------------------------
        int lx[3] = { 0, 0, 0 };   // old nearest node, tile-local
        T dlt[3] = { T( 0 ), T( 0 ), T( 0 ) };
        int gnode[3] = { 0, 0, 0 };
        int img[3] = { 0, 0, 0 }; // FP64 form: N when the old node was wrapped to its image 0
        double xabs[3] = { 0.0, 0.0, 0.0 };
        double xpn[3] = { 0.0, 0.0, 0.0 };
        T px = T( 0 ), py = T( 0 ), pz = T( 0 ), w = T( 0 ), tauv = T( 0 );
        if( valid && in.tau ) {
            if constexpr( CELLS ) tauv = ( T )sRec[6 * nmax + q];
            else tauv = in.tau[src];
        }
        if( valid ) {
            if constexpr( CELLS ) {
                // slot q of the cell-ordered planes
                const int lc = sSlotCell[q];
                if( DIM == 3 ) {
                    gnode[0] = ix0 + lc / ( g.T[1] * g.T[2] );
                    gnode[1] = iy0 + ( lc / g.T[2] ) % g.T[1];
                    gnode[2] = iz0 + lc % g.T[2];
                } else {
                    gnode[0] = ix0 + lc / g.T[1];
                    gnode[1] = iy0 + lc % g.T[1];
                }
#pragma unroll
                for( int d = 0; d < DIM; d++ ) dlt[d] = ( T )sRec[d * nmax + q];
            } else if constexpr( MIXED ) {
                const unsigned key = in.key[src];
                unpack_key( DIM, key, gnode[0], gnode[1], gnode[2] );
#pragma unroll
                for( int d = 0; d < DIM; d++ ) dlt[d] = ( T )in.d[d][src];
            } else {
#pragma unroll
                for( int d = 0; d < DIM; d++ ) {
                    xabs[d] = ( double )in.x[d][src];
                    xpn[d] = xabs[d] * g.dxi[d];
                    int ip = round_half_away( xpn[d] );
                    if( !g.open[d] && ip >= g.N[d] ) { // periodic, x in [L - dx/2, L): use the image node 0
                        ip -= g.N[d];
                        img[d] = g.N[d];
                        xpn[d] -= ( double )g.N[d];
                    }
                    gnode[d] = ip;
                    dlt[d] = ( T )( xpn[d] - ( double )ip );
                }
            }
            if constexpr( CELLS ) {
                px = ( T )sRec[3 * nmax + q];
                py = ( T )sRec[4 * nmax + q];
                pz = ( T )sRec[5 * nmax + q];
                w = ( T )sRec[7 * nmax + q];
            } else {
                px = ( T )in.p[0][src];
                py = ( T )in.p[1][src];
                pz = ( T )in.p[2][src];
                w = ( T )in.w[src];
            }
        }
        lx[0] = gnode[0] - ix0;
        lx[1] = gnode[1] - iy0;
        lx[2] = DIM == 3 ? gnode[2] - iz0 : 0;
        const bool inside = lx[0] >= 0 && lx[0] < g.T[0] && lx[1] >= 0 && lx[1] < g.T[1] &&
                            ( DIM == 2 || ( lx[2] >= 0 && lx[2] < g.T[2] ) );
        if( valid && !inside ) atomicCAS( status, 0, SG_ERR_BOUNDS );
        // lanes past the tile's last particle, and particles found outside the
        // tile, read the tile at its origin: every shared-memory index stays in range
        if( !valid || !inside ) lx[0] = lx[1] = lx[2] = 0;

        // ---- gather ---------------------------------------------------------------
        T cp[3][3], cd[3][3];
        int sd[3] = { 0, 0, 0 };
#pragma unroll
        for( int d = 0; d < 3; d++ ) {
            if( d < DIM ) {
                bspline2( dlt[d], cp[d][0], cp[d][1], cp[d][2] );
                T dd;
                if constexpr( MIXED ) {
                    sd[d] = dlt[d] >= T( 0 ) ? 1 : 0;
                    dd = dlt[d] + T( 0.5 ) - T( sd[d] );
                } else {
                    const int id = round_half_away( xpn[d] + 0.5 );
                    sd[d] = id - gnode[d];
                    dd = ( T )( xpn[d] - ( double )id + 0.5 );
                }
                bspline2( dd, cd[d][0], cd[d][1], cd[d][2] );
            } else {
                cp[d][0] = cp[d][2] = T( 0 ); cp[d][1] = T( 1 );
                cd[d][0] = cd[d][2] = T( 0 ); cd[d][1] = T( 1 );
            }
        }
        // clamp the dual shift for safety (0 or 1 by construction)
#pragma unroll
        for( int d = 0; d < 3; d++ ) sd[d] = sd[d] < 0 ? 0 : ( sd[d] > 1 ? 1 : sd[d] );
        // (TMA's box starts one z node lower)
        const int bz_p = DIM == 3 ? lx[2] + ( TMA ? 1 : 0 ) : 0, bz_d = DIM == 3 ? lx[2] + sd[2] + ( TMA ? 1 : 0 ) : 0;
        const int bx_p = lx[0], bx_d = lx[0] + sd[0], by_p = lx[1], by_d = lx[1] + sd[1];
        // Ex(d,p,p) Ey(p,d,p) Ez(p,p,d) Bx(p,d,d) By(d,p,d) Bz(d,d,p)
        T Ex, Ey, Ez, Bx, By, Bz;
        if constexpr( MIXED ) {
            // paired: (Ex, By) share their x and y windows, (Ey, Bx) too
            const float2 exby = gather_pair<DIM>( sF + 0 * fsz, sF + 4 * fsz, td, cd[0], cd[0], cp[1], cp[1], cp[2], cd[2],
                                                  bx_d, by_p, bz_p, bx_d, by_p, bz_d );
            const float2 eybx = gather_pair<DIM>( sF + 1 * fsz, sF + 3 * fsz, td, cp[0], cp[0], cd[1], cd[1], cp[2], cd[2],
                                                  bx_p, by_d, bz_p, bx_p, by_d, bz_d );
            const float2 ezbz = gather_pair<DIM>( sF + 2 * fsz, sF + 5 * fsz, td, cp[0], cd[0], cp[1], cd[1], cd[2], cp[2],
                                                  bx_p, by_p, bz_d, bx_d, by_d, bz_p );
            Ex = exby.x; By = exby.y;
            Ey = eybx.x; Bx = eybx.y;
            Ez = ezbz.x; Bz = ezbz.y;
        } else {
            Ex = gather_tile<DIM, T>( sF + 0 * fsz, td, cd[0], cp[1], cp[2], bx_d, by_p, bz_p );
            Ey = gather_tile<DIM, T>( sF + 1 * fsz, td, cp[0], cd[1], cp[2], bx_p, by_d, bz_p );
            Ez = gather_tile<DIM, T>( sF + 2 * fsz, td, cp[0], cp[1], cd[2], bx_p, by_p, bz_d );
            Bx = gather_tile<DIM, T>( sF + 3 * fsz, td, cp[0], cd[1], cd[2], bx_p, by_d, bz_d );
            By = gather_tile<DIM, T>( sF + 4 * fsz, td, cd[0], cp[1], cd[2], bx_d, by_p, bz_d );
            Bz = gather_tile<DIM, T>( sF + 5 * fsz, td, cd[0], cd[1], cp[2], bx_d, by_d, bz_p );
        }

        // ---- push -----------------------------------------------------------------
        const T ginv = push_t<KIND, T>( qm, Ex, Ey, Ez, Bx, By, Bz, px, py, pz );

        // ---- move: new position, node shift per dimension ---------------------
        int shift[3] = { 0, 0, 0 };
        T dnew[3] = { T( 0 ), T( 0 ), T( 0 ) };
        const T pm[3] = { px, py, pz };
        if constexpr( MIXED ) {
#pragma unroll
            for( int d = 0; d < DIM; d++ ) {
                const T dn = dlt[d] + pm[d] * ( ginv * vs[d] );
                const int sh = ( int )floorf( ( float )dn + 0.5f );
                shift[d] = sh;
                dnew[d] = dn - T( sh );
            }
        } else {
#pragma unroll
            for( int d = 0; d < DIM; d++ ) {
                double xn;
                if( KIND == 0 ) xn = xabs[d] + ( double )pm[d] * ( ( double )ginv * g.dt );
                else xn = xabs[d] + g.dt * ( double )pm[d] * ( double )ginv;
                xabs[d] = xn;
                // same image shift as the old position (exact: both terms are near N)
                const double xnn = xn * g.dxi[d] - ( double )img[d];
                const int ipn = round_half_away( xnn );
                shift[d] = ipn - gnode[d];
                dnew[d] = ( T )( xnn - ( double )ipn );
            }
        }
        bool moved_ok = true;
#pragma unroll
        for( int d = 0; d < DIM; d++ ) {
            if( shift[d] < -1 || shift[d] > 1 ) moved_ok = false;
        }
        if( valid && !moved_ok ) {
            atomicCAS( status, 0, SG_ERR_BOUNDS );
#pragma unroll
            for( int d = 0; d < DIM; d++ ) shift[d] = shift[d] < -1 ? -1 : ( shift[d] > 1 ? 1 : shift[d] );
        }
        // leaving through an open boundary (x < 0 or x >= L): the particle loses its charge
        // and deposits nothing (remove_particle_inf/_sup, BoundaryConditionType.cpp:204-294)
        bool gone = false;
#pragma unroll
        for( int d = 0; d < DIM; d++ ) {
            if( !g.open[d] ) continue;
            if constexpr( MIXED ) {
                const int v = gnode[d] + shift[d];
                gone |= v < 0 || ( v == 0 && dnew[d] < T( 0 ) ) || v > g.N[d] || ( v == g.N[d] && dnew[d] >= T( 0 ) );
            } else {
                gone |= xabs[d] < 0.0 || xabs[d] >= g.L[d];
            }
        }
        gone = gone && valid;

        // ---- Esirkepov deposit: direct, or a record for the per-cell pass ----
        if( valid ) {
            if constexpr( CELLS ) {
                const int sbits = gone ? GONE_RECORD : ( shift[0] + 1 ) | ( ( shift[1] + 1 ) << 2 ) | ( ( shift[2] + 1 ) << 4 );
                sRec[3 * nmax + q] = ( float )dnew[0];
                sRec[4 * nmax + q] = ( float )dnew[1];
                sRec[5 * nmax + q] = DIM == 3 ? ( float )dnew[2] : ( float )( pz * ginv );
                sRec[6 * nmax + q] = __int_as_float( sbits );
            } else if( !gone ) {
                EsirWin<T> W[3];
#pragma unroll
                for( int d = 0; d < DIM; d++ ) {
                    // the old weights of the deposit (the gather's, requantised in the mixed form)
                    T o0 = cp[d][0], o1 = cp[d][1], o2 = cp[d][2];
                    if constexpr( MIXED ) dep_spline( dlt[d], o0, o1, o2 );
                    esir_win<T>( o0, o1, o2, dnew[d], shift[d], W[d] );
                }
                const T cr[3] = { cr3[0] * w, cr3[1] * w, cr3[2] * w };
                deposit_direct<DIM, T>( sJ, td, jsz, lx, W, cr, cw0 * w * pz * ginv );
            }
        }

        if constexpr( CELLS ) {
            // node-changing particles go to a list deposited with full warps later (3D: the
            // per-cell pass takes their footprint part, the list the planes beyond it)
            const int nshift = ( shift[0] != 0 ) + ( shift[1] != 0 ) + ( shift[2] != 0 );
            const bool cross = valid && !gone && nshift > 0;
            if( cross ) atomicAdd( &sXc[nshift == 1 ? ( shift[0] != 0 ? 0 : ( shift[1] != 0 ? 1 : 2 ) ) : 3], 1 );
            const unsigned xm = __ballot_sync( 0xffffffffu, cross );
            if( xm ) {
                int xb = 0;
                if( lane == 0 ) xb = atomicAdd( &sNX, __popc( xm ) );
                xb = __shfl_sync( 0xffffffffu, xb, 0 );
                if( cross ) sRank[xb + __popc( xm & ( ( 1u << lane ) - 1u ) )] = q;
            }
        }

        // ---- destination tile and write-out --------------------------------------
        // periodic axes wrap; an open axis keeps nodes 0..N (particles beyond are gone)
        int nn[3] = { 0, 0, 0 };
        if constexpr( MIXED ) {
#pragma unroll
            for( int d = 0; d < DIM; d++ ) {
                int v = gnode[d] + shift[d];
                if( !g.open[d] ) {
                    if( v < 0 ) v += g.N[d];
                    if( v >= g.N[d] ) v -= g.N[d];
                }
                nn[d] = v;
            }
        } else {
#pragma unroll
            for( int d = 0; d < DIM; d++ ) {
                double x = xabs[d];
                if( !g.open[d] ) {
                    if( x < 0.0 ) x += g.L[d];
                    if( x >= g.L[d] ) x -= g.L[d];
                }
                xabs[d] = x;
                int ip = round_half_away( x * g.dxi[d] );
                if( !g.open[d] && ip >= g.N[d] ) ip -= g.N[d];
                nn[d] = ip;
            }
        }
        const bool keep = valid && !gone;
        // a non-finite or runaway particle must not index outside the tile tables
#pragma unroll
        for( int d = 0; d < DIM; d++ ) {
            if( keep && ( nn[d] < 0 || nn[d] >= g.N[d] + g.open[d] ) ) {
                atomicCAS( status, 0, SG_ERR_BOUNDS );
                nn[d] = 0;
            }
        }
        {
            const unsigned gm = __ballot_sync( 0xffffffffu, gone );
            if( gm && lane == 0 ) atomicAdd( removed, __popc( gm ) );
        }
        const int dest = keep ? tile_of( g, nn[0], nn[1], DIM == 3 ? nn[2] : 0 ) : -1;
        // warp-aggregated slot allocation per destination tile
        const unsigned peers = __match_any_sync( 0xffffffffu, dest );
        const int leader = __ffs( peers ) - 1;
        int slot_base = 0;
        if( keep && ( int )lane == leader ) slot_base = atomicAdd( &count_out[dest], __popc( peers ) );
        slot_base = __shfl_sync( 0xffffffffu, slot_base, leader );
        if( keep ) {
            const int slot = slot_base + __popc( peers & ( ( 1u << lane ) - 1u ) );
            PBuf<MIXED> dst = out;
            int64_t o;
            if( slot < cap[dest] ) {
                o = seg_start[dest] + slot;
            } else {
                const int k = atomicAdd( ovf_count, 1 );
                if( k >= ovf_cap ) {
                    atomicCAS( status, 0, SG_ERR_OVERFLOW );
                    o = -1;
                } else {
                    dst = ovf;
                    o = k;
                    ovf_tile[k] = dest;
                }
            }
            if( o >= 0 ) {
                if constexpr( MIXED ) {
                    dst.key[o] = pack_key( DIM, nn[0], nn[1], nn[2] );
#pragma unroll
                    for( int d = 0; d < DIM; d++ ) dst.d[d][o] = ( float )dnew[d];
                } else {
#pragma unroll
                    for( int d = 0; d < DIM; d++ ) dst.x[d][o] = xabs[d];
                }
                dst.p[0][o] = px;
                dst.p[1][o] = py;
                dst.p[2][o] = pz;
                dst.w[o] = w;
                if( dst.tau ) dst.tau[o] = tauv;
            }
        }
    }
    __syncthreads();

    if constexpr( CELLS ) {
        // group the node-changing list by class (counting sort), each class from a warp
        // boundary; class starts in sXc, the padding slots hold -1
        if( threadIdx.x == 0 ) {
            int run = 0;
            for( int k = 0; k < 4; k++ ) {
                const int c = sXc[k];
                sXn[k] = c;
                sXb[k] = run;
                sXc[k] = run;
                run += ( c + 31 ) & ~31;
            }
            sNT = run;
        }
        __syncthreads();
        for( int i = threadIdx.x; i < 128; i += blockDim.x ) {
            const int k = i >> 5, l = i & 31;
            if( l < ( ( sXn[k] + 31 ) & ~31 ) - sXn[k] ) sXs[sXb[k] + sXn[k] + l] = -1;
        }
        for( int k = threadIdx.x; k < sNX; k += blockDim.x ) {
            const int q = sRank[k];
            const int sb = __float_as_int( sRec[6 * nmax + q] );
            const int h0 = ( sb & 3 ) - 1, h1 = ( ( sb >> 2 ) & 3 ) - 1, h2 = ( ( sb >> 4 ) & 3 ) - 1;
            const int nsh = ( h0 != 0 ) + ( h1 != 0 ) + ( h2 != 0 );
            const int cls = nsh == 1 ? ( h0 != 0 ? 0 : ( h1 != 0 ? 1 : 2 ) ) : 3;
            sXs[atomicAdd( &sXc[cls], 1 )] = q;
        }
        __syncthreads();
    }

    // 3. per-cell deposit (CELLS).  Particles that stay on their node in every
    // dimension share their cell's fixed footprint: stencil points 1..3 across the
    // current, 2..3 along it (point 4 carries a sum that is exactly zero).  Their
    // contributions are summed in registers and added once per cell.  In 3D so is the
    // footprint part of a particle that changes node in one dimension (its new weights
    // moved by the shift); the node-changing pass adds the plane beyond.  Particles
    // that change node in more dimensions (3D) or at all (2D) are deposited directly
    // (into sJ2).  3D: thread
    // t works on cell t % TC, group j = t / TC; even groups own Jx and the lower
    // Jz plane, odd groups Jy and the upper one; groups j>>1 split the records.
    // 2D: the groups split the records and own all three components.
    if constexpr( CELLS ) {
        // groups per cell (even in 3D: the two halves of the footprint pair up)
        const int tpc = DIM == 3 ? ( ( int )( blockDim.x / TC ) & ~1 ) : ( int )( blockDim.x / TC );
        const int c = threadIdx.x % TC, grp = threadIdx.x / TC;
        if( grp < tpc ) {
            int cl[3];
            if( DIM == 3 ) {
                cl[2] = c % g.T[2];
                cl[1] = ( c / g.T[2] ) % g.T[1];
                cl[0] = c / ( g.T[2] * g.T[1] );
            } else {
                cl[2] = 0;
                cl[1] = c % g.T[1];
                cl[0] = c / g.T[1];
            }
            const T twelfth = T( 1.0 / 12.0 );
            const int hf = DIM == 3 ? ( grp & 1 ) : 0;
            const int q0 = DIM == 3 ? ( grp >> 1 ) : grp, qstep = DIM == 3 ? ( tpc >> 1 ) : tpc;
            // 3D: acc = along-axis current (m, u, v), accz = Jz plane hf (u, v)
            // 2D: acc = Jx (m, u) then Jy (u, m), accz = Jz (u, v)
            T acc[18], accz[9];
            float2 acc2[9]; // 3D: the along-axis current's two planes (m = 0, 1) as a pair
#pragma unroll
            for( int k = 0; k < 18; k++ ) acc[k] = T( 0 );
#pragma unroll
            for( int k = 0; k < 9; k++ ) {
                accz[k] = T( 0 );
                acc2[k] = make_float2( 0.f, 0.f );
            }
            const int end = sStart[c] + sCnt[c];
            for( int q = sStart[c] + q0; q < end; q += qstep ) {
                const int sb = __float_as_int( sRec[6 * nmax + q] );
                int sh[3] = { 0, 0, 0 };
                if constexpr( DIM == 3 ) {
                    // every particle: one that changes node adds its footprint part here
                    // (the node-changing pass the rest); a removed one deposits nothing
                    if( sb == GONE_RECORD ) continue;
                    sh[0] = ( sb & 3 ) - 1;
                    sh[1] = ( ( sb >> 2 ) & 3 ) - 1;
                    sh[2] = ( ( sb >> 4 ) & 3 ) - 1;
                } else {
                    if( sb != NO_SHIFT ) continue; // in the node-changing list
                }
                T dold[3], dn[3];
                dold[0] = sRec[q];
                dold[1] = sRec[nmax + q];
                dold[2] = DIM == 3 ? sRec[2 * nmax + q] : T( 0 );
                dn[0] = sRec[3 * nmax + q];
                dn[1] = sRec[4 * nmax + q];
                dn[2] = DIM == 3 ? sRec[5 * nmax + q] : T( 0 );
                const T vz = DIM == 3 ? T( 0 ) : sRec[5 * nmax + q];
                const T wq = sRec[7 * nmax + q];
                const T cr[3] = { cr3[0] * wq, cr3[1] * wq, cr3[2] * wq };
                {
                    T A[3][3], D[3][3], P[3][2];
                    if constexpr( DIM == 3 ) {
                        T nov[3]; // (the node-changing pass deposits the plane beyond the footprint)
                        footprint_weights3<T>( dold, dn, sh, A, D, P, nov );
                    } else if constexpr( MIXED ) {
                        T nov[3];
                        footprint_weights_xy( dold, dn, sh, A, D, P, nov );
                    } else {
#pragma unroll
                        for( int d = 0; d < DIM; d++ ) {
                            T nov;
                            footprint_weights<T>( dold[d], dn[d], sh[d], A[d], D[d], P[d], nov );
                        }
                    }
                    if( DIM == 3 ) {
                        // along-axis a = hf, transverse b = 1 - hf and 2
                        const T cra = hf ? cr[1] : cr[0];
                        const T pa0 = hf ? P[1][0] : P[0][0], pa1 = hf ? P[1][1] : P[0][1];
                        const T pz = hf ? P[2][1] : P[2][0];
                        // paired FP32 arithmetic (FFMA2): (wt, wz) together, then both planes
                        // of the along-axis current in one instruction
                        const float2 cpa = make_float2( -( cra * pa0 ), -( cra * pa1 ) );
                        const T cpz = -( cr[2] * pz );
#pragma unroll
                        for( int u = 0; u < 3; u++ ) {
                            const T ab = hf ? A[0][u] : A[1][u], db = hf ? D[0][u] : D[1][u];
                            const float2 au = make_float2( ab, A[0][u] ), du = make_float2( twelfth * db, twelfth * D[0][u] );
#pragma unroll
                            for( int v = 0; v < 3; v++ ) {
                                // .x = wt = ab A_z + db D_z / 12, .y = wz = A_x A_y + D_x D_y / 12
                                const float2 w2 = __ffma2_rn( au, make_float2( A[2][v], A[1][v] ),
                                                              __fmul2_rn( du, make_float2( D[2][v], D[1][v] ) ) );
                                acc2[u * 3 + v] = __ffma2_rn( cpa, make_float2( w2.x, w2.x ), acc2[u * 3 + v] );
                                accz[u * 3 + v] = fmaf( cpz, w2.y, accz[u * 3 + v] );
                            }
                        }
                    } else {
                        const T crz = cw0 * wq * vz;
#pragma unroll
                        for( int u = 0; u < 3; u++ ) {
#pragma unroll
                            for( int m = 0; m < 2; m++ ) {
                                acc[m * 3 + u] -= cr[0] * P[0][m] * A[1][u];
                                acc[6 + u * 2 + m] -= cr[1] * P[1][m] * A[0][u];
                            }
#pragma unroll
                            for( int v = 0; v < 3; v++ ) accz[u * 3 + v] += crz * ( A[0][u] * A[1][v] + twelfth * D[0][u] * D[1][v] );
                        }
                    }
                }
            }
            if( DIM == 3 ) {
                T *Ja = sJ + hf * jsz, *Jz = sJ + 2 * jsz;
#pragma unroll
                for( int u = 0; u < 3; u++ )
#pragma unroll
                    for( int v = 0; v < 3; v++ ) {
#pragma unroll
                        for( int m = 0; m < 2; m++ ) {
                            const int ia = ( hf ? cl[0] + 1 + u : cl[0] + 2 + m ), ib = ( hf ? cl[1] + 2 + m : cl[1] + 1 + u );
                            const int ea = ia * td.JXS + ib * td.JZ + cl[2] + 1 + v;
                            sh_add( &Ja[ea], m == 0 ? acc2[u * 3 + v].x : acc2[u * 3 + v].y );
                        }
                        const int ez = ( cl[0] + 1 + u ) * td.JXS + ( cl[1] + 1 + v ) * td.JZ + cl[2] + 2 + hf;
                        sh_add( &Jz[ez], accz[u * 3 + v] );
                    }
            } else {
                T *J0 = sJ, *J1 = sJ + jsz, *J2 = sJ + 2 * jsz;
#pragma unroll
                for( int u = 0; u < 3; u++ ) {
#pragma unroll
                    for( int m = 0; m < 2; m++ ) {
                        const int e0 = ( cl[0] + 2 + m ) * td.JXS + cl[1] + 1 + u, e1 = ( cl[0] + 1 + u ) * td.JXS + cl[1] + 2 + m;
                        sh_add( &J0[e0], acc[m * 3 + u] );
                        sh_add( &J1[e1], acc[6 + u * 2 + m] );
                    }
#pragma unroll
                    for( int v = 0; v < 3; v++ ) {
                        const int e2 = ( cl[0] + 1 + u ) * td.JXS + cl[1] + 1 + v;
                        sh_add( &J2[e2], accz[u * 3 + v] );
                    }
                }
            }
        }
        // node-changing particles, one per thread, into their own tile (after the
        // per-cell pass: warps that finish their cells early start on this list)
        for( int k = threadIdx.x; k < sNT; k += blockDim.x ) {
            const int q = sXs[k];
            if( q < 0 ) continue; // padding
            const int lc = sSlotCell[q];
            int cl[3];
            if( DIM == 3 ) {
                cl[2] = lc % g.T[2];
                cl[1] = ( lc / g.T[2] ) % g.T[1];
                cl[0] = lc / ( g.T[2] * g.T[1] );
            } else {
                cl[2] = 0;
                cl[1] = lc % g.T[1];
                cl[0] = lc / g.T[1];
            }
            const int sbits = __float_as_int( sRec[6 * nmax + q] );
            const int sh[3] = { ( sbits & 3 ) - 1, ( ( sbits >> 2 ) & 3 ) - 1, ( ( sbits >> 4 ) & 3 ) - 1 };
            const T wq = sRec[7 * nmax + q];
            const T cr[3] = { cr3[0] * wq, cr3[1] * wq, cr3[2] * wq };
            if constexpr( DIM == 3 ) {
                // the per-cell pass took the footprint part, this the planes beyond
                T A[3][3], D[3][3], P[3][2], nov[3];
                const T dq_old[3] = { ( T )sRec[q], ( T )sRec[nmax + q], ( T )sRec[2 * nmax + q] };
                const T dq_new[3] = { ( T )sRec[3 * nmax + q], ( T )sRec[4 * nmax + q], ( T )sRec[5 * nmax + q] };
                footprint_weights3<T>( dq_old, dq_new, sh, A, D, P, nov );
                deposit_beyond<T>( sJ2, jsz, td.JXS, td.JZ, cl, A, D, P, cr, nov, sh );
                continue;
            }
            const T vz = DIM == 3 ? T( 0 ) : sRec[5 * nmax + q];
            EsirWin<T> W[3];
#pragma unroll
            for( int d = 0; d < DIM; d++ ) {
                T o0, o1, o2;
                dep_spline( ( T )sRec[d * nmax + q], o0, o1, o2 );
                esir_win<T>( o0, o1, o2, ( T )sRec[( 3 + d ) * nmax + q], sh[d], W[d] );
            }
            // the list is grouped by crossing dimension, so a warp's zero nodes mostly coincide
            const T crz = cw0 * wq * vz;
            deposit_direct<DIM, T>( sJ2, td, jsz, cl, W, cr, crz );
        }
        // the list's reads of the field tile come before the next staging's writes
        if constexpr( TMA ) asm volatile( "fence.proxy.async.shared::cta;\n" ::: "memory" );
        __syncthreads();
    }
    } // chunk
    // a tile without particles still waits for its field copies before the CTA ends
    if constexpr( CELLS ) cp_async_wait_all();
    if constexpr( TMA ) {
        if( tma_pending ) {
            tma_wait( &sTmaBar, tma_phase, status );
            tma_phase ^= 1u;
            tma_pending = false;
        }
    }

    // 4. flush the J tile (origin = array index i0 + OS - 2) with global atomics
    const TileMap jm = tile_map<DIM>( td.JY, td.JZ );
#pragma unroll
    for( int c = 0; c < 3; c++ ) {
        double *dstJ = f.J[c];
        const int ny = ext( g, 1, stag( c, 1 ) ), nz = ext( g, 2, stag( c, 2 ) );
        const int nx = ext( g, 0, stag( c, 0 ) );
        const T *srcJ = sJ + c * jsz, *srcJ2 = sJ2 + c * jsz;
        if( jm.fast ) {
            if( jm.active ) {
                const int gy = iy0 + OS - 2 + jm.cy, gz = DIM == 3 ? iz0 + OS - 2 + jm.cz : 0;
                for( int cx = jm.cx0; cx < td.JX; cx += jm.step ) {
                    const int e = cx * td.JXS + jm.cy * td.JZ + jm.cz;
                    const T v = tile_value<CELLS, T>( srcJ, srcJ2, e );
                    const int gx = ix0 + OS - 2 + cx;
                    if( v != T( 0 ) && gx < nx && gy < ny && gz < nz )
                        atomicAdd( &dstJ[( ( int64_t )gx * ny + gy ) * nz + gz], to_global( v ) );
                }
            }
        } else {
            for( int e = threadIdx.x; e < jsz; e += blockDim.x ) {
                const T v = tile_value<CELLS, T>( srcJ, srcJ2, e );
                if( v == T( 0 ) ) continue;
                const int cx = e / td.JXS, r = e - cx * td.JXS, cy = r / td.JZ, cz = r - cy * td.JZ;
                const int gx = ix0 + OS - 2 + cx, gy = iy0 + OS - 2 + cy, gz = DIM == 3 ? iz0 + OS - 2 + cz : 0;
                if( cy < td.JY && gx < nx && gy < ny && gz < nz ) atomicAdd( &dstJ[( ( int64_t )gx * ny + gy ) * nz + gz], to_global( v ) );
            }
        }
    }
    if( !sp.queue ) break;
    } // tile
}

// ------------------------------------------------------------------------------
// Field kernels of the periodic single-grid step.
// ------------------------------------------------------------------------------

// dst rows of nz4 values (zeros past nz) from src rows of nz: the padded layout the TMA
// tensor maps need (rows a multiple of 16 bytes).  One thread per padded value.
__global__ void k_pad_rows( const float *__restrict__ src, float *__restrict__ dst, int64_t rows, int nz, int nz4 )
{
    const int64_t n = rows * nz4;
    for( int64_t t = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x; t < n; t += ( int64_t )gridDim.x * blockDim.x ) {
        const int64_t r = t / nz4;
        const int k = ( int )( t - r * nz4 );
        dst[t] = k < nz ? src[r * nz + k] : 0.0f;
    }
}

// Periodic J ghost fold along dimension d (the same-process branch of
// SyncVectorPatch::sumAllComponents, SyncVectorPatch.cpp:203-330): the first
// 1 + 2*OS (+1 if dual) planes and their images N planes further are summed and
// both set to the sum.  blockIdx.y = component.
template <class T>
__global__ void k_fold( GridInfo g, int d, Fields<T> f )
{
    const int c = blockIdx.y;
    double *a = f.J[c];
    const int e0 = ext( g, 0, stag( c, 0 ) ), e1 = ext( g, 1, stag( c, 1 ) ), e2 = ext( g, 2, stag( c, 2 ) );
    int se[3] = { e0, e1, e2 };
    se[d] = 1 + 2 * OS + stag( c, d );
    const int64_t n = ( int64_t )se[0] * se[1] * se[2];
    for( int64_t t = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x; t < n; t += ( int64_t )gridDim.x * blockDim.x ) {
        const int k = ( int )( t % se[2] );
        const int j = ( int )( ( t / se[2] ) % se[1] );
        const int i = ( int )( t / ( ( int64_t )se[2] * se[1] ) );
        int i2 = i, j2 = j, k2 = k;
        if( d == 0 ) i2 += g.N[0];
        else if( d == 1 ) j2 += g.N[1];
        else k2 += g.N[2];
        const int64_t a1 = ( ( int64_t )i * e1 + j ) * e2 + k;
        const int64_t a2 = ( ( int64_t )i2 * e1 + j2 ) * e2 + k2;
        const double v = a[a2] + a[a1];
        a[a2] = v;
        a[a1] = v;
    }
}

// Ampere on every point (MA_Solver3D_norm.cpp:18-115 / MA_Solver2D_norm.cpp:18-107).
// One block per row of the last dimension; E stays consistent between a node and
// its periodic image because J (folded) and B (synchronised) are.

// Error-free transforms (Knuth's two-sum, the FMA two-product): a + b = s + e and
// a * b = p + e exactly in floating point.
template <class T>
__device__ __forceinline__ void two_sum( T a, T b, T &s, T &e )
{
    s = a + b;
    const T bb = s - a;
    e = ( a - ( s - bb ) ) + ( b - bb );
}
template <class T>
__device__ __forceinline__ void two_prod( T a, T b, T &p, T &e )
{
    p = a * b;
    e = fma( a, b, -p );
}

// Ampere increment of one E point: -dt J + ca (b1 - b0) + cb (b3 - b2) (cb = 0: one curl
// term).  FP64 form: plain arithmetic in the reference's order.  Mixed form (C given):
// the increment is formed exactly as a pair (hi + lo) with error-free transforms, and E
// is kept as the pair E - C (C the compensation), so an Ampere step adds no rounding
// of its own to E: div E follows div J and the discrete curl of B exactly (the curl
// part cancels in the divergence whatever B is).
// The padded copies of E (p[0..2]) and B_m (p[3..5]) that the TMA tensor maps read:
// rows of nz4[c] floats, a multiple of 16 bytes.  The field kernels write them beside
// the arrays (null pointers: no TMA staging).
struct PadOut {
    float *p[6];
    int nz4[6];
};

// FP64 to an FP32 pair hi + lo with integer operations: hi is d with its fraction cut
// to 23 bits, lo the next 24 bits of the rest (hi + lo is d to about 2^-47 relative for
// |d| above 2^-98; below, lo is 0).  Magnitudes beyond the FP32 range give +-infinity
// (NaN stays NaN), below 2^-126 +-0.
__device__ __forceinline__ void split_fp64( double d, float &hi, float &lo )
{
    const unsigned long long b = ( unsigned long long )__double_as_longlong( d );
    const unsigned sgn = ( unsigned )( b >> 32 ) & 0x80000000u;
    const int e = ( int )( ( b >> 52 ) & 0x7ffu ) - 1023;
    const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
    lo = 0.f;
    if( e > 127 ) {
        hi = __uint_as_float( sgn | 0x7f800000u | ( e == 1024 && m ? 0x400000u : 0u ) );
        return;
    }
    if( e < -126 ) {
        hi = __uint_as_float( sgn );
        return;
    }
    hi = __uint_as_float( sgn | ( ( unsigned )( e + 127 ) << 23 ) | ( unsigned )( m >> 29 ) );
    const unsigned low = ( unsigned )( m & 0x1FFFFFFFull );
    if( low == 0u ) return;
    const int p = 31 - __clz( low ), fe = e - 52 + p;
    if( fe < -126 ) return;
    const unsigned frac = ( p >= 23 ? low >> ( p - 23 ) : low << ( 23 - p ) ) & 0x7fffffu;
    lo = __uint_as_float( sgn | ( ( unsigned )( fe + 127 ) << 23 ) | frac );
}

template <class T>
__device__ __forceinline__ T ampere_point( T *E, T *C, int64_t t, T dt, double Jd, T ca, T b1, T b0, T cb, T b3, T b2 )
{
    if( !C ) {
        const T J = ( T )Jd;
        const T En = E[t] + ( -dt * J + ca * ( b1 - b0 ) + cb * ( b3 - b2 ) );
        E[t] = En;
        return En;
    }
    // the FP64 current as an FP32 pair J + Jl (integer operations: FP64 conversions and
    // adds take this GPU's FP64 pipe, 1/64 of the FP32 rate)
    T J, Jl;
    if constexpr( sizeof( T ) == 4 ) split_fp64( Jd, J, Jl );
    else {
        J = ( T )Jd;
        Jl = T( 0 );
    }
    T d1, e1, d2, e2, p1, q1, p2, q2, p3, q3, s, es, S, eS;
    two_sum( b1, -b0, d1, e1 );
    two_sum( b3, -b2, d2, e2 );
    two_prod( -dt, J, p1, q1 );
    q1 += -dt * Jl;
    two_prod( ca, d1, p2, q2 );
    two_prod( cb, d2, p3, q3 );
    two_sum( p1, p2, s, es );
    two_sum( s, p3, S, eS );
    const T lo = ( ( q1 + q2 ) + ( q3 + ca * e1 ) ) + ( ( cb * e2 + es ) + eS );
    T Es, eE;
    two_sum( E[t], S, Es, eE );
    const T low = ( eE + lo ) - C[t];
    const T En = Es + low;
    C[t] = ( En - Es ) - low;
    E[t] = En;
    return En;
}

template <int DIM, class T>
__global__ void k_ampere_all( GridInfo g, Fields<T> f, T dt, T dtdx, T dtdy, T dtdz, PadOut po )
{
    const int nxp = g.np[0], nyp = g.np[1], nyd = nyp + 1;
    if( DIM == 3 ) {
        const int nzp = g.np[2], nzd = nzp + 1;
        const int row = blockIdx.x; // over (nxp + 1) * nyd
        const int i = row / nyd, j = row % nyd;
        for( int k = threadIdx.x; k < nzd; k += blockDim.x ) {
            if( j < nyp && k < nzp ) {
                const int64_t r = ( int64_t )i * nyp + j, t = r * nzp + k;
                const T e = ampere_point( f.E[0], f.Ec[0], t, dt, f.J[0][t], dtdy, f.B[2][( ( int64_t )i * nyd + j + 1 ) * nzp + k], f.B[2][( ( int64_t )i * nyd + j ) * nzp + k],
                                          -dtdz, f.B[1][( ( int64_t )i * nyp + j ) * nzd + k + 1], f.B[1][( ( int64_t )i * nyp + j ) * nzd + k] );
                if constexpr( sizeof( T ) == 4 )
                    if( po.p[0] ) po.p[0][r * po.nz4[0] + k] = e;
            }
            if( i < nxp && k < nzp ) {
                const int64_t r = ( int64_t )i * nyd + j, t = r * nzp + k;
                const T e = ampere_point( f.E[1], f.Ec[1], t, dt, f.J[1][t], -dtdx, f.B[2][( ( int64_t )( i + 1 ) * nyd + j ) * nzp + k], f.B[2][t],
                                          dtdz, f.B[0][( ( int64_t )i * nyd + j ) * nzd + k + 1], f.B[0][( ( int64_t )i * nyd + j ) * nzd + k] );
                if constexpr( sizeof( T ) == 4 )
                    if( po.p[1] ) po.p[1][r * po.nz4[1] + k] = e;
            }
            if( i < nxp && j < nyp ) {
                const int64_t r = ( int64_t )i * nyp + j, t = r * nzd + k;
                const T e = ampere_point( f.E[2], f.Ec[2], t, dt, f.J[2][t], dtdx, f.B[1][( ( int64_t )( i + 1 ) * nyp + j ) * nzd + k], f.B[1][t],
                                          -dtdy, f.B[0][( ( int64_t )i * nyd + j + 1 ) * nzd + k], f.B[0][( ( int64_t )i * nyd + j ) * nzd + k] );
                if constexpr( sizeof( T ) == 4 )
                    if( po.p[2] ) po.p[2][r * po.nz4[2] + k] = e;
            }
        }
    } else {
        const int i = blockIdx.x; // over nxd
        for( int j = threadIdx.x; j < nyd; j += blockDim.x ) {
            if( j < nyp ) {
                const int64_t t = ( int64_t )i * nyp + j;
                ampere_point( f.E[0], f.Ec[0], t, dt, f.J[0][t], dtdy, f.B[2][( int64_t )i * nyd + j + 1], f.B[2][( int64_t )i * nyd + j], T( 0 ), T( 0 ), T( 0 ) );
            }
            if( i < nxp ) {
                const int64_t t = ( int64_t )i * nyd + j;
                ampere_point( f.E[1], f.Ec[1], t, dt, f.J[1][t], -dtdx, f.B[2][( int64_t )( i + 1 ) * nyd + j], f.B[2][t], T( 0 ), T( 0 ), T( 0 ) );
            }
            if( i < nxp && j < nyp ) {
                const int64_t t = ( int64_t )i * nyp + j;
                ampere_point( f.E[2], f.Ec[2], t, dt, f.J[2][t], dtdx, f.B[1][( int64_t )( i + 1 ) * nyp + j], f.B[1][t],
                              -dtdy, f.B[0][( int64_t )i * nyd + j + 1], f.B[0][( int64_t )i * nyd + j] );
            }
        }
    }
}

// Periodic image of a dual index in the outermost layers (0 -> N, nd-1 -> nd-1-N).
__device__ __forceinline__ int canon( int i, int nd, int N ) { return i == 0 ? N : ( i == nd - 1 ? i - N : i ); }

// Faraday on every point (MF_Solver3D_Yee.cpp:18-111 on the interior; the
// outermost dual layers take their periodic image's update, which is what the
// reference's B exchange copies there), fused with the B_m centring
// (ElectroMagn3D::centerMagneticFields, ElectroMagn3D.cpp:1191): B_m = (B_new + B_old)/2.
// ---- open boundaries (2D) ---------------------------------------------------

// Faraday on a 2D grid with open axes (MF_Solver2D_Yee::operator(),
// MF_Solver2D_Yee.cpp:18-140): along an open axis only interior points are
// updated (the boundary layer is left to the Silver-Mueller condition); along a
// periodic one every point is, the outermost dual layer from its periodic image.
// B_m receives the old B everywhere (saveMagneticFields).  One thread per point
// of the (nxd x nyd) box.
template <class T>
__global__ void k_faraday_open2d( GridInfo g, Fields<T> f, T dtdx, T dtdy )
{
    const int nxp = g.np[0], nyp = g.np[1], nxd = nxp + 1, nyd = nyp + 1;
    const int64_t t = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x;
    if( t >= ( int64_t )nxd * nyd ) return;
    const int x = ( int )( t / nyd ), y = ( int )( t % nyd );
    const int lox = g.open[0] ? 1 : 0, hix = g.open[0] ? nxd - 1 : nxd;
    const int loy = g.open[1] ? 1 : 0, hiy = g.open[1] ? nyd - 1 : nyd;
    const int xc = g.open[0] ? x : canon( x, nxd, g.N[0] ), yc = g.open[1] ? y : canon( y, nyd, g.N[1] );
    const T *Ex = f.E[0], *Ey = f.E[1], *Ez = f.E[2];
    if( x < nxp ) { // Bx (p,d)
        const int64_t i = ( int64_t )x * nyd + y;
        const T old = f.B[0][i];
        f.Bm[0][i] = old;
        if( y >= loy && y < hiy ) f.B[0][i] = old - dtdy * ( Ez[x * nyp + yc] - Ez[x * nyp + yc - 1] );
    }
    if( y < nyp ) { // By (d,p)
        const int64_t i = ( int64_t )x * nyp + y;
        const T old = f.B[1][i];
        f.Bm[1][i] = old;
        if( x >= lox && x < hix ) f.B[1][i] = old + dtdx * ( Ez[( int64_t )xc * nyp + y] - Ez[( int64_t )( xc - 1 ) * nyp + y] );
    }
    { // Bz (d,d)
        const int64_t i = ( int64_t )x * nyd + y;
        const T old = f.B[2][i];
        f.Bm[2][i] = old;
        if( x >= lox && x < hix && y >= loy && y < hiy )
            f.B[2][i] = old + dtdy * ( Ex[( int64_t )x * nyp + yc] - Ex[( int64_t )x * nyp + yc - 1] )
                        - dtdx * ( Ey[( int64_t )xc * nyd + y] - Ey[( int64_t )( xc - 1 ) * nyd + y] );
    }
}

// Gaussian 2D laser on xmin, in the terms of the reference's LaserGaussian2D
// (pyprofiles.py:507-569, transformPolarization :458-468), time envelope tgaussian
// (Function.cpp:528-535); amplitude of LaserProfileSeparable::getAmplitude
// (Laser.cpp:453-460).  FP64.
struct LaserG2 {
    double omega, fy, invWaist2, coeff, sqrtw, amp[2], delay[2], phase_offset;
    double t_start, t_end, t_center, t_invsigma, t_order;
};

__device__ inline double laser_amp( const LaserG2 &L, int profile, double y, double t )
{
    const double dy = y - L.fy;
    const double S = L.amp[profile] * L.sqrtw * exp( -L.invWaist2 * dy * dy );
    const double phi = L.coeff * dy * dy - L.phase_offset + L.delay[profile == 0 ? 1 : 0];
    const double tt = t - ( phi + L.delay[profile] ) / L.omega;
    const double env = ( tt < L.t_start || tt > L.t_end ) ? 0.0 : exp( -pow( tt - L.t_center, L.t_order ) * L.t_invsigma );
    return env * S * sin( L.omega * t - phi );
}

constexpr int MAX_LASERS = 4;
struct OpenBC {
    double coef[4][5];      // Silver-Mueller Alpha..Epsilon per side (xmin, xmax, ymin, ymax)
    int side_mask;          // bit s: side s is applied (the x sides are skipped when the window moves)
    int nlaser;             // lasers on xmin
    LaserG2 laser[MAX_LASERS];
};

// Silver-Mueller on every open side of a 2D grid (ElectroMagnBC2D_SM::apply,
// ElectroMagnBC2D_SM.cpp:118-265, no external fields), the lasers on xmin at
// time_dual = (step + 1.5) dt.  The four sides write disjoint points and read
// no point another side writes, so one launch covers them: blockIdx.y = side.
template <class T>
__global__ void k_silver_mueller2d( GridInfo g, Fields<T> f, OpenBC bc, const int64_t *__restrict__ step )
{
    const int side = blockIdx.y, ax = side / 2, tan = ax == 0 ? 1 : 0;
    if( !g.open[ax] || !( ( bc.side_mask >> side ) & 1 ) ) return;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int nxp = g.np[0], nyp = g.np[1], nyd = nyp + 1;
    const int mx = side % 2, sgn = mx ? 1 : -1;
    const int np0 = g.np[ax], nd0 = np0 + 1;
    int iB[3];
    if( !mx ) {
        iB[0] = iB[1] = iB[2] = 0;
    } else {
        iB[ax] = np0 - 1;
        iB[tan] = nd0 - 1;
        iB[2] = nd0 - 1;
    }
    const int p0 = iB[0] - sgn, p1 = iB[1] - sgn, p2 = iB[2] - sgn;
    const int tmin = g.open[tan], tmax = g.open[tan];
    const int n1p = g.np[tan], n1d = n1p + 1;
    const double Al = bc.coef[side][0], Be = bc.coef[side][1], Ga = bc.coef[side][2], De = bc.coef[side][3],
                 Ep = bc.coef[side][4];
    const double t = ( ( double )*step + 1.5 ) * g.dt;
    const T *Ex = f.E[0], *Ey = f.E[1], *Ez = f.E[2];
    T *Bx = f.B[0], *By = f.B[1], *Bz = f.B[2];
    if( j >= tmin && j < n1p - tmax ) {
        double b1 = 0.0;
        if( side == 0 )
            for( int k = 0; k < bc.nlaser; k++ ) b1 += laser_amp( bc.laser[k], 0, ( j - OS ) * g.dx[1], t );
        if( ax == 0 )
            By[( int64_t )iB[1] * nyp + j] = ( T )( Al * Ez[( int64_t )iB[0] * nyp + j] + Be * By[( int64_t )p1 * nyp + j] + Ga * b1
                                                    + De * Bx[( int64_t )iB[0] * nyd + j + 1] + Ep * Bx[( int64_t )iB[0] * nyd + j] );
        else
            Bx[iB[0] + ( int64_t )nyd * j] = ( T )( -Al * Ez[iB[1] + ( int64_t )nyp * j] + Be * Bx[p0 + ( int64_t )nyd * j] + Ga * b1
                                                     + De * By[iB[1] + ( int64_t )nyp * ( j + 1 )] + Ep * By[iB[1] + ( int64_t )nyp * j] );
    }
    if( j >= tmin && j < n1d - tmax ) {
        double b2 = 0.0;
        if( side == 0 )
            for( int k = 0; k < bc.nlaser; k++ ) b2 += laser_amp( bc.laser[k], 1, ( j - 0.5 - OS ) * g.dx[1], t );
        if( ax == 0 )
            Bz[( int64_t )iB[2] * nyd + j] = ( T )( -Al * Ey[( int64_t )iB[0] * nyd + j] + Be * Bz[( int64_t )p2 * nyd + j] + Ga * b2 );
        else
            Bz[( int64_t )j * nyd + iB[2]] = ( T )( Al * Ex[( int64_t )j * nyp + iB[1]] + Be * Bz[( int64_t )j * nyd + p2] + Ga * b2 );
    }
    ( void )nxp;
}

// B_m <- (B + B_m)/2 on every point (centerMagneticFields); block 0 advances the
// step counter the boundary lasers read.
template <class T>
__global__ void k_center_b2d( GridInfo g, Fields<T> f, int64_t *__restrict__ step )
{
    const int nxp = g.np[0], nyp = g.np[1], nxd = nxp + 1, nyd = nyp + 1;
    const int64_t t = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x;
    if( t == 0 ) *step += 1;
    if( t >= ( int64_t )nxd * nyd ) return;
    const int x = ( int )( t / nyd ), y = ( int )( t % nyd );
    if( x < nxp ) f.Bm[0][t] = ( f.B[0][t] + f.Bm[0][t] ) * T( 0.5 );
    if( y < nyp ) {
        const int64_t i = ( int64_t )x * nyp + y;
        f.Bm[1][i] = ( f.B[1][i] + f.Bm[1][i] ) * T( 0.5 );
    }
    f.Bm[2][t] = ( f.B[2][t] + f.Bm[2][t] ) * T( 0.5 );
}

template <int DIM, class T>
__global__ void k_faraday_center( GridInfo g, Fields<T> f, T dtdx, T dtdy, T dtdz, PadOut po )
{
    const int nxp = g.np[0], nyp = g.np[1], nxd = nxp + 1, nyd = nyp + 1;
    const int Nx = g.N[0], Ny = g.N[1];
    if( DIM == 3 ) {
        const int nzp = g.np[2], nzd = nzp + 1, Nz = g.N[2];
        const int row = blockIdx.x;
        const int i = row / nyd, j = row % nyd;
        const T *Ex = f.E[0], *Ey = f.E[1], *Ez = f.E[2];
        for( int k = threadIdx.x; k < nzd; k += blockDim.x ) {
            if( i < nxp ) { // Bx(p,d,d)
                const int jc = canon( j, nyd, Ny ), kc = canon( k, nzd, Nz );
                const int64_t t = ( ( int64_t )i * nyd + j ) * nzd + k;
                const T old = f.B[0][t];
                const T nw = old + ( -dtdy * ( Ez[( ( int64_t )i * nyp + jc ) * nzd + k] - Ez[( ( int64_t )i * nyp + jc - 1 ) * nzd + k] )
                                     + dtdz * ( Ey[( ( int64_t )i * nyd + j ) * nzp + kc] - Ey[( ( int64_t )i * nyd + j ) * nzp + kc - 1] ) );
                f.B[0][t] = nw;
                const T bm = ( nw + old ) * T( 0.5 );
                f.Bm[0][t] = bm;
                if constexpr( sizeof( T ) == 4 )
                    if( po.p[3] ) po.p[3][( ( int64_t )i * nyd + j ) * po.nz4[3] + k] = bm;
            }
            if( j < nyp ) { // By(d,p,d)
                const int ic = canon( i, nxd, Nx ), kc = canon( k, nzd, Nz );
                const int64_t t = ( ( int64_t )i * nyp + j ) * nzd + k;
                const T old = f.B[1][t];
                const T nw = old + ( -dtdz * ( Ex[( ( int64_t )i * nyp + j ) * nzp + kc] - Ex[( ( int64_t )i * nyp + j ) * nzp + kc - 1] )
                                     + dtdx * ( Ez[( ( int64_t )ic * nyp + j ) * nzd + k] - Ez[( ( int64_t )( ic - 1 ) * nyp + j ) * nzd + k] ) );
                f.B[1][t] = nw;
                const T bm = ( nw + old ) * T( 0.5 );
                f.Bm[1][t] = bm;
                if constexpr( sizeof( T ) == 4 )
                    if( po.p[4] ) po.p[4][( ( int64_t )i * nyp + j ) * po.nz4[4] + k] = bm;
            }
            if( k < nzp ) { // Bz(d,d,p)
                const int ic = canon( i, nxd, Nx ), jc = canon( j, nyd, Ny );
                const int64_t t = ( ( int64_t )i * nyd + j ) * nzp + k;
                const T old = f.B[2][t];
                const T nw = old + ( -dtdx * ( Ey[( ( int64_t )ic * nyd + j ) * nzp + k] - Ey[( ( int64_t )( ic - 1 ) * nyd + j ) * nzp + k] )
                                     + dtdy * ( Ex[( ( int64_t )i * nyp + jc ) * nzp + k] - Ex[( ( int64_t )i * nyp + jc - 1 ) * nzp + k] ) );
                f.B[2][t] = nw;
                const T bm = ( nw + old ) * T( 0.5 );
                f.Bm[2][t] = bm;
                if constexpr( sizeof( T ) == 4 )
                    if( po.p[5] ) po.p[5][( ( int64_t )i * nyd + j ) * po.nz4[5] + k] = bm;
            }
        }
    } else {
        const int i = blockIdx.x;
        const T *Ex = f.E[0], *Ey = f.E[1], *Ez = f.E[2];
        for( int j = threadIdx.x; j < nyd; j += blockDim.x ) {
            if( i < nxp ) { // Bx(p,d)
                const int jc = canon( j, nyd, Ny );
                const int64_t t = ( int64_t )i * nyd + j;
                const T old = f.B[0][t];
                const T nw = old - dtdy * ( Ez[( int64_t )i * nyp + jc] - Ez[( int64_t )i * nyp + jc - 1] );
                f.B[0][t] = nw;
                f.Bm[0][t] = ( nw + old ) * T( 0.5 );
            }
            if( j < nyp ) { // By(d,p)
                const int ic = canon( i, nxd, Nx );
                const int64_t t = ( int64_t )i * nyp + j;
                const T old = f.B[1][t];
                const T nw = old + dtdx * ( Ez[( int64_t )ic * nyp + j] - Ez[( int64_t )( ic - 1 ) * nyp + j] );
                f.B[1][t] = nw;
                f.Bm[1][t] = ( nw + old ) * T( 0.5 );
            }
            { // Bz(d,d)
                const int ic = canon( i, nxd, Nx ), jc = canon( j, nyd, Ny );
                const int64_t t = ( int64_t )i * nyd + j;
                const T old = f.B[2][t];
                const T nw = old + ( dtdy * ( Ex[( int64_t )i * nyp + jc] - Ex[( int64_t )i * nyp + jc - 1] )
                                     - dtdx * ( Ey[( int64_t )ic * nyd + j] - Ey[( int64_t )( ic - 1 ) * nyd + j] ) );
                f.B[2][t] = nw;
                f.Bm[2][t] = ( nw + old ) * T( 0.5 );
            }
        }
    }
}

// ------------------------------------------------------------------------------
// Layout kernels (initial placement and re-layout after a spill; not per step).
// ------------------------------------------------------------------------------

// From FP64 positions/momenta/weights to the form's state; records the tile and counts it.
template <int DIM, bool MIXED>
__global__ void k_stage( GridInfo g, int64_t n, const double *__restrict__ pos, const double *__restrict__ mom,
                         const double *__restrict__ wgt, PBuf<MIXED> st, int *__restrict__ st_tile,
                         int *__restrict__ count )
{
    const int64_t p = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x;
    if( p >= n ) return;
    int node[3] = { 0, 0, 0 };
#pragma unroll
    for( int d = 0; d < DIM; d++ ) {
        double x = pos[d * n + p];
        if( !g.open[d] ) {
            if( x < 0.0 ) x += g.L[d];
            if( x >= g.L[d] ) x -= g.L[d];
        }
        const double xn = x * g.dxi[d];
        int ip = round_half_away( xn );
        double dl = xn - ( double )ip;
        if( g.open[d] ) {
            // positions on an open axis must lie in [0, L): nodes 0..N
            if( ip < 0 || ip > g.N[d] ) ip = 0;
        } else {
            if( ip >= g.N[d] ) ip -= g.N[d];
            if( ip < 0 ) ip += g.N[d];
            if( ip < 0 || ip >= g.N[d] ) ip = 0; // non-finite input: keep the index inside the tables
        }
        node[d] = ip;
        if constexpr( MIXED ) st.d[d][p] = ( float )dl;
        else st.x[d][p] = x;
    }
    using PT = typename std::conditional<MIXED, float, double>::type;
    if constexpr( MIXED ) st.key[p] = pack_key( DIM, node[0], node[1], node[2] );
    st.p[0][p] = ( PT )mom[p];
    st.p[1][p] = ( PT )mom[n + p];
    st.p[2][p] = ( PT )mom[2 * n + p];
    st.w[p] = ( PT )wgt[p];
    if( st.tau ) st.tau[p] = ( PT )-1.0;
    const int t = tile_of( g, node[0], node[1], node[2] );
    st_tile[p] = t;
    atomicAdd( &count[t], 1 );
}

// cap[t] = count[t] + max(count[t] * slack, slack * (largest count of the face
// neighbours), min_extra), rounded up to a multiple of 4.  The neighbour term
// gives a sparse tile next to a dense one room for the particles that flow in,
// so density edges do not spill every step.
__global__ void k_caps( GridInfo g, const int *__restrict__ count, int *__restrict__ cap, float slack, int min_extra )
{
    const int nt = g.ntiles;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if( t >= nt ) return;
    const int n2 = g.ndim == 3 ? g.nt[2] : 1, n1 = g.nt[1], n0 = g.nt[0];
    const int tz = t % n2, ty = ( t / n2 ) % n1, tx = t / ( n2 * n1 );
    int nb = 0;
    for( int d = 0; d < g.ndim; d++ )
        for( int sgn = -1; sgn <= 1; sgn += 2 ) {
            int x = tx, y = ty, z = tz;
            if( d == 0 ) x = ( tx + sgn + n0 ) % n0;
            if( d == 1 ) y = ( ty + sgn + n1 ) % n1;
            if( d == 2 ) z = ( tz + sgn + n2 ) % n2;
            nb = max( nb, count[( x * n1 + y ) * n2 + z] );
        }
    const int c = count[t];
    const int v = c + max( max( ( int )ceilf( c * slack ), ( int )ceilf( nb * slack ) ), min_extra );
    cap[t] = ( v + 3 ) & ~3;
}

template <bool MIXED>
__device__ __forceinline__ void copy_particle( const PBuf<MIXED> &s, int64_t i, const PBuf<MIXED> &d, int64_t o,
                                               int ndim )
{
    if constexpr( MIXED ) {
        d.key[o] = s.key[i];
        for( int k = 0; k < ndim; k++ ) d.d[k][o] = s.d[k][i];
    } else {
        for( int k = 0; k < ndim; k++ ) d.x[k][o] = s.x[k][i];
    }
    d.p[0][o] = s.p[0][i];
    d.p[1][o] = s.p[1][i];
    d.p[2][o] = s.p[2][i];
    d.w[o] = s.w[i];
    if( s.tau ) d.tau[o] = s.tau[i];
}

// Staged (or spilled) particle -> next free slot of its tile in the destination buffer.
// Thread t places particle (t * 2654435761) mod n, a permutation of [0, n) (the
// multiplier is a prime above 2^31 > n): inputs usually arrive cell by cell, and
// scrambling them inside each tile keeps the lanes of a warp on different cells,
// which is what keeps the deposit's shared-memory atomics free of conflicts.
template <bool MIXED>
__global__ void k_place( int ndim, int64_t n, PBuf<MIXED> st, const int *__restrict__ st_tile,
                         const int64_t *__restrict__ seg_start, int *__restrict__ fill, PBuf<MIXED> dst )
{
    const int64_t th = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x;
    if( th >= n ) return;
    // th < 2^31 and the multiplier < 2^32: the product fits in 64 bits
    const int64_t p = ( int64_t )( ( ( unsigned long long )th * 2654435761ull ) % ( unsigned long long )n );
    const int t = st_tile[p];
    const int slot = atomicAdd( &fill[t], 1 );
    copy_particle<MIXED>( st, p, dst, seg_start[t] + slot, ndim );
}

// Re-layout: the live part of every old segment is copied to the new segment; fill = copied count.
template <bool MIXED>
__global__ void k_relayout_tiles( int ndim, int nt, const int64_t *__restrict__ old_start,
                                  const int *__restrict__ old_cap, const int *__restrict__ count, PBuf<MIXED> src,
                                  const int64_t *__restrict__ new_start, PBuf<MIXED> dst, int *__restrict__ fill )
{
    const int t = blockIdx.x;
    if( t >= nt ) return;
    const int n = min( count[t], old_cap[t] );
    for( int i = threadIdx.x; i < n; i += blockDim.x )
        copy_particle<MIXED>( src, old_start[t] + i, dst, new_start[t] + i, ndim );
    if( threadIdx.x == 0 ) fill[t] = n;
}

// ------------------------------------------------------------------------------
// Moving window (SimWindow::shift, src/MovWindow/SimWindow.cpp:98-560) and
// particle creation from a density profile (ParticleCreator::create,
// src/Particles/ParticleCreator.cpp:110-345).  The reference drops its xmin patch
// and appends a zeroed patch at xmax, keeping absolute particle positions; here
// the one grid keeps its place and its contents move `shift` cells towards xmin.
// These run on the (rare) steps at which the window moves, outside the graphs.
// ------------------------------------------------------------------------------

// dst[i] = src[i + shift] for the points in front of the fresh region, 0 in it;
// one thread per point, x the slowest index (plane = points per x index).
template <class T>
__global__ void k_window_shift_field( const T *__restrict__ src, T *__restrict__ dst, int64_t ex, int64_t plane,
                                      int64_t keep, int shift )
{
    const int64_t n = ex * plane;
    for( int64_t t = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x; t < n; t += ( int64_t )gridDim.x * blockDim.x ) {
        const int64_t i = t / plane;
        dst[t] = i < keep ? src[t + ( int64_t )shift * plane] : T( 0 );
    }
}

// Nearest node of an FP64 position, as the initial placement computes it.
__device__ __forceinline__ int node_fp64( const GridInfo &g, double x, int d )
{
    int ip = round_half_away( x * g.dxi[d] );
    if( g.open[d] ) {
        if( ip < 0 || ip > g.N[d] ) ip = 0;
    } else {
        if( ip >= g.N[d] ) ip -= g.N[d];
        if( ip < 0 ) ip += g.N[d];
        if( ip < 0 || ip >= g.N[d] ) ip = 0;
    }
    return ip;
}

// Every live particle moves `shift` cells towards xmin in place (mixed form: the
// x node of the key, exact; FP64 form: x -= shift dx); one now at x < 0 lay in
// the dropped cells and is removed (slot_tile = -1).  Else slot_tile = its tile,
// counted in newcount.  shift = 0 only re-bins.  One block per tile.
template <int DIM, bool MIXED>
__global__ void k_window_particles( GridInfo g, const int64_t *__restrict__ seg_start, const int *__restrict__ count,
                                    PBuf<MIXED> b, int shift, int *__restrict__ slot_tile, int *__restrict__ newcount,
                                    unsigned long long *__restrict__ removed )
{
    const int t = blockIdx.x;
    const int n = count[t];
    const int64_t s0 = seg_start[t];
    unsigned gone_here = 0;
    for( int i = threadIdx.x; i < n; i += blockDim.x ) {
        const int64_t o = s0 + i;
        int node[3] = { 0, 0, 0 };
        bool gone;
        if constexpr( MIXED ) {
            unpack_key( DIM, b.key[o], node[0], node[1], node[2] );
            node[0] -= shift;
            gone = node[0] < 0 || ( node[0] == 0 && b.d[0][o] < 0.0f );
            if( !gone ) b.key[o] = pack_key( DIM, node[0], node[1], node[2] );
        } else {
            const double x = b.x[0][o] - ( double )shift * g.dx[0];
            gone = x < 0.0;
            b.x[0][o] = x;
#pragma unroll
            for( int d = 0; d < DIM; d++ ) node[d] = node_fp64( g, b.x[d][o], d );
        }
        if( gone ) {
            slot_tile[o] = -1;
            gone_here++;
        } else {
            const int nt = tile_of( g, node[0], node[1], node[2] );
            slot_tile[o] = nt;
            atomicAdd( &newcount[nt], 1 );
        }
    }
    if( gone_here ) atomicAdd( removed, ( unsigned long long )gone_here );
}

// Survivors of k_window_particles -> next free slot of their tile in dst.
template <bool MIXED>
__global__ void k_window_place( int ndim, const int64_t *__restrict__ seg_start, const int *__restrict__ count,
                                PBuf<MIXED> src, const int *__restrict__ slot_tile, const int64_t *__restrict__ new_start,
                                int *__restrict__ fill, PBuf<MIXED> dst )
{
    const int t = blockIdx.x;
    const int n = count[t];
    const int64_t s0 = seg_start[t];
    for( int i = threadIdx.x; i < n; i += blockDim.x ) {
        const int64_t o = s0 + i;
        const int nt = slot_tile[o];
        if( nt < 0 ) continue;
        const int slot = atomicAdd( &fill[nt], 1 );
        copy_particle<MIXED>( src, o, dst, new_start[nt] + slot, ndim );
    }
}

// Density profile and particle layout of created plasma.
struct InjectParams {
    double prof[5];      // n0, x_vacuum, x_slope1, x_plateau, x_slope2 (trapezoidal in x)
    double vol;          // cell volume
    double invc;         // 1 / particles per cell per dimension
    double sqrt_temp;    // sqrt(temperature); 0: cold
    unsigned long long seed;
    long long n_moved;   // cells the window has moved: absolute cell = n_moved + window cell
    int ppc, c;          // particles per cell = c^ndim
    int x0, x1;          // window cells [x0, x1) along x, every cell along y (z)
};

// trapeze (src/Profiles/Function.cpp:291-310)
__device__ inline double trapeze( double x, double plateau, double slope1, double slope2 )
{
    double r = 0.0;
    if( x > 0.0 ) {
        if( x < slope1 ) {
            r = x / slope1;
        } else {
            x -= slope1 + plateau;
            if( x < 0.0 ) {
                r = 1.0;
            } else {
                x -= slope2;
                if( x < 0.0 ) r = -x / slope2;
            }
        }
    }
    return r;
}

// splitmix64 output function (Steele, Lea and Flood 2014) over a key of
// (seed, absolute cell, draw): each particle's momentum draw is independent of
// the order in which particles are created.
__device__ __forceinline__ unsigned long long mix64( unsigned long long z )
{
    z += 0x9E3779B97F4A7C15ull;
    z = ( z ^ ( z >> 30 ) ) * 0xBF58476D1CE4E5B9ull;
    z = ( z ^ ( z >> 27 ) ) * 0x94D049BB133111EBull;
    return z ^ ( z >> 31 );
}

__device__ __forceinline__ double uniform_open0( unsigned long long seed, unsigned long long cell, unsigned long long k )
{
    const unsigned long long h = mix64( mix64( seed ^ mix64( cell ) ) + k );
    return ( double )( ( h >> 11 ) + 1 ) * ( 1.0 / 9007199254740992.0 ); // (0, 1]
}

// One thread per cell of the region.  pass 0 counts the new particles per tile
// (newcount, created); pass 1 writes them to the next free slots of their tiles
// (fill, new_start) of dst.  Regular positions x = i dx + dx 0.975 / c (0.5 + m)
// (ParticleCreator::createPosition, ParticleCreator.cpp:661-667), weight
// n(x_centre) dV / ppc (createWeight, :933-939); rounded products and sums (no
// contraction) so that positions and weights are those of the FP64 restatement.
template <int DIM, bool MIXED>
__global__ void k_inject( GridInfo g, InjectParams ip, int pass, int *__restrict__ newcount,
                          unsigned long long *__restrict__ created, const int64_t *__restrict__ new_start,
                          int *__restrict__ fill, PBuf<MIXED> dst )
{
    const int ny = g.N[1], nz = DIM == 3 ? g.N[2] : 1;
    const int64_t ncell = ( int64_t )( ip.x1 - ip.x0 ) * ny * nz;
    const int64_t cidx = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x;
    if( cidx >= ncell ) return;
    const int k = ( int )( cidx % nz ), j = ( int )( ( cidx / nz ) % ny ), i = ip.x0 + ( int )( cidx / ( ( int64_t )ny * nz ) );
    const double xc = __dmul_rn( ( double )( ip.n_moved + i ) + 0.5, g.dx[0] );
    const double dens = __dmul_rn( ip.prof[0], trapeze( __dadd_rn( xc, -ip.prof[1] ), ip.prof[3], ip.prof[2], ip.prof[4] ) );
    if( !( dens > 0.0 ) ) return;
    const double w = __dmul_rn( dens, ip.vol ) / ( double )ip.ppc;
    const int ci[3] = { i, j, k };
    const unsigned long long cell =
        ( ( unsigned long long )( ip.n_moved + i ) * ( unsigned long long )ny + ( unsigned long long )j ) * ( unsigned long long )nz + ( unsigned long long )k;
    for( int p = 0; p < ip.ppc; p++ ) {
        double x[3] = { 0.0, 0.0, 0.0 };
        int node[3] = { 0, 0, 0 };
        int m = p;
#pragma unroll
        for( int d = 0; d < DIM; d++ ) {
            const double off = __dmul_rn( __dmul_rn( __dmul_rn( g.dx[d], 0.975 ), ip.invc ), 0.5 + ( double )( m % ip.c ) );
            x[d] = __dadd_rn( __dmul_rn( ( double )ci[d], g.dx[d] ), off );
            m /= ip.c;
            node[d] = node_fp64( g, x[d], d );
        }
        const int t = tile_of( g, node[0], node[1], node[2] );
        if( pass == 0 ) {
            atomicAdd( &newcount[t], 1 );
            continue;
        }
        double pm[3] = { 0.0, 0.0, 0.0 };
        if( ip.sqrt_temp > 0.0 ) {
            const unsigned long long base = ( unsigned long long )p * 4ull;
            const double r1 = sqrt( -2.0 * log( uniform_open0( ip.seed, cell, base ) ) );
            const double a1 = 6.283185307179586 * uniform_open0( ip.seed, cell, base + 1 );
            const double r2 = sqrt( -2.0 * log( uniform_open0( ip.seed, cell, base + 2 ) ) );
            const double a2 = 6.283185307179586 * uniform_open0( ip.seed, cell, base + 3 );
            pm[0] = ip.sqrt_temp * r1 * cos( a1 );
            pm[1] = ip.sqrt_temp * r1 * sin( a1 );
            pm[2] = ip.sqrt_temp * r2 * cos( a2 );
        }
        const int slot = atomicAdd( &fill[t], 1 );
        const int64_t o = new_start[t] + slot;
        if constexpr( MIXED ) {
            dst.key[o] = pack_key( DIM, node[0], node[1], node[2] );
#pragma unroll
            for( int d = 0; d < DIM; d++ ) { // offset from the nearest node before a periodic wrap
                const double xn = __dmul_rn( x[d], g.dxi[d] );
                dst.d[d][o] = ( float )( xn - ( double )round_half_away( xn ) );
            }
        } else {
#pragma unroll
            for( int d = 0; d < DIM; d++ ) dst.x[d][o] = x[d];
        }
        using PT = typename std::conditional<MIXED, float, double>::type;
        dst.p[0][o] = ( PT )pm[0];
        dst.p[1][o] = ( PT )pm[1];
        dst.p[2][o] = ( PT )pm[2];
        dst.w[o] = ( PT )w;
        if( dst.tau ) dst.tau[o] = ( PT )-1.0;
    }
    if( pass == 0 ) atomicAdd( created, ( unsigned long long )ip.ppc );
}

// ------------------------------------------------------------------------------
// FP64 reductions for the energy diagnostics.
// ------------------------------------------------------------------------------
__device__ __forceinline__ double block_sum( double v )
{
    __shared__ double red[32];
#pragma unroll
    for( int o = 16; o > 0; o >>= 1 ) v += __shfl_down_sync( 0xffffffffu, v, o );
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if( lane == 0 ) red[warp] = v;
    __syncthreads();
    v = threadIdx.x < ( blockDim.x >> 5 ) ? red[threadIdx.x] : 0.0;
    if( warp == 0 ) {
#pragma unroll
        for( int o = 16; o > 0; o >>= 1 ) v += __shfl_down_sync( 0xffffffffu, v, o );
    }
    return v;
}

// sum over live particles of w * (gamma - 1) (DiagnosticScalar.cpp:505-522): a warp per
// tile at a time, each lane summing its share of the tile (a contiguous segment) and
// adding that to its FP64 total once per tile.
template <bool MIXED>
__global__ void k_kinetic( int nt, const int64_t *__restrict__ seg_start, const int *__restrict__ count,
                           PBuf<MIXED> b, double *__restrict__ out )
{
    const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    double acc = 0.0;
    for( int t = blockIdx.x * wpb + ( threadIdx.x >> 5 ); t < nt; t += gridDim.x * wpb ) {
        const int n = count[t];
        const int64_t s0 = seg_start[t];
        if constexpr( MIXED ) {
            // FP32 momenta: gamma - 1 = p^2 / (1 + gamma) in FP32 (no cancellation at small p),
            // a lane's terms of the tile (about n / 32) summed in FP32, then in FP64
            float part = 0.0f;
#pragma unroll 4
            for( int i = lane; i < n; i += 32 ) {
                const float px = b.p[0][s0 + i], py = b.p[1][s0 + i], pz = b.p[2][s0 + i];
                const float p2 = fmaf( px, px, fmaf( py, py, pz * pz ) );
                part = fmaf( b.w[s0 + i], p2 / ( 1.0f + sqrtf( 1.0f + p2 ) ), part );
            }
            acc += ( double )part;
        } else {
#pragma unroll 4
            for( int i = lane; i < n; i += 32 ) {
                const double px = b.p[0][s0 + i], py = b.p[1][s0 + i], pz = b.p[2][s0 + i];
                acc += b.w[s0 + i] * ( sqrt( 1.0 + px * px + py * py + pz * pz ) - 1.0 );
            }
        }
    }
    acc = block_sum( acc );
    if( threadIdx.x == 0 ) atomicAdd( out, acc );
}

// sum of w and of w (gamma - 1) over one species (the scalar diagnostics' Dens and Ukin).
template <bool MIXED>
__global__ void k_species_sums( int nt, const int64_t *__restrict__ seg_start, const int *__restrict__ count,
                                PBuf<MIXED> b, double *__restrict__ out )
{
    double sw = 0.0, se = 0.0;
    for( int t = blockIdx.x; t < nt; t += gridDim.x ) {
        const int n = count[t];
        const int64_t s0 = seg_start[t];
        for( int i = threadIdx.x; i < n; i += blockDim.x ) {
            const double px = b.p[0][s0 + i], py = b.p[1][s0 + i], pz = b.p[2][s0 + i];
            const double w = b.w[s0 + i];
            sw += w;
            se += w * ( sqrt( 1.0 + px * px + py * py + pz * pz ) - 1.0 );
        }
    }
    sw = block_sum( sw );
    se = block_sum( se );
    if( threadIdx.x == 0 ) {
        atomicAdd( out, sw );
        atomicAdd( out + 1, se );
    }
}

// Six field arrays for k_norm2: pointers and their extents along dimensions 1 and 2.
struct Norm2Set {
    const void *a[6];
    int e1[6], e2[6];
};

// sum of F^2 over the N physical points per dimension (array index OS .. OS+N-1) of array
// blockIdx.y of `f`, into out[blockIdx.y * per_array]: a warp per row of the last
// dimension at a time, each lane summing its points of the row in the field's type and
// adding that to its FP64 total once per row.
template <class T>
__global__ void k_norm2( GridInfo g, Norm2Set f, int per_array, double *__restrict__ out )
{
    const T *__restrict__ a = static_cast<const T *>( f.a[blockIdx.y] );
    const int e1 = f.e1[blockIdx.y], e2 = f.e2[blockIdx.y];
    const bool d3 = g.ndim == 3;
    const int nrow = d3 ? g.N[0] * g.N[1] : g.N[0], len = d3 ? g.N[2] : g.N[1];
    const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    double acc = 0.0;
    for( int r = blockIdx.x * wpb + ( threadIdx.x >> 5 ); r < nrow; r += gridDim.x * wpb ) {
        int64_t base;
        if( d3 ) {
            const int i = r / g.N[1], j = r - i * g.N[1];
            base = ( ( int64_t )( i + OS ) * e1 + ( j + OS ) ) * e2 + OS;
        } else {
            base = ( int64_t )( r + OS ) * e1 + OS;
        }
        T part = T( 0 );
#pragma unroll 4
        for( int k = lane; k < len; k += 32 ) {
            const T v = a[base + k];
            part = fma( v, v, part );
        }
        acc += ( double )part;
    }
    acc = block_sum( acc );
    if( threadIdx.x == 0 ) atomicAdd( out + blockIdx.y * per_array, acc );
}

__global__ void k_bump_step( int64_t *step ) { *step += 1; }

// PusherPhoton::operator() (src/Pusher/PusherPhoton.cpp:30-85) on a species' stored
// macro-photons (2D, FP64 planes of cap values): x += dt p / |p|, then the periodic wrap
// on periodic axes (length L[d]; BoundaryConditionType.cpp periodic).  The count of
// stored photons is read on the device: min(*count, cap).
__global__ void k_push_resident_photons( int64_t cap, const unsigned long long *__restrict__ count, double dt,
                                         double *__restrict__ pos, const double *__restrict__ mom, double L0,
                                         double L1, int periodic0, int periodic1 )
{
    const int64_t n = min( ( int64_t )*count, cap );
    for( int64_t k = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x; k < n; k += ( int64_t )gridDim.x * blockDim.x ) {
        const double px = mom[k], py = mom[cap + k], pz = mom[2 * cap + k];
        const double inv = 1.0 / sqrt( px * px + py * py + pz * pz );
        double x = pos[k] + dt * px * inv, y = pos[cap + k] + dt * py * inv;
        if( periodic0 ) x = x < 0.0 ? x + L0 : ( x >= L0 ? x - L0 : x );
        if( periodic1 ) y = y < 0.0 ? y + L1 : ( y >= L1 ? y - L1 : y );
        pos[k] = x;
        pos[cap + k] = y;
    }
}

// Steps in one batched graph.
constexpr int BATCH_STEPS = 8;

// Ints of the batch record: [0] stop, [1] steps done, [2] step limit (from the host),
// [3 + s] particles removed from species s over the batch, then the flags of the last
// step done (1 + 2 * max_species ints, layout of d_flags).
__host__ __device__ constexpr int batch_record_ints( int max_species ) { return 3 + max_species + 1 + 2 * max_species; }

// Gate k of a batched graph (one thread): accounts for step k - 1 if it ran (its removals
// summed, its flags kept; a spill or an error stops the batch) and, unless it is the last
// gate, sets the condition of step k's node: run while not stopped and k < the limit.
// Gate 0 clears the record.  The flags are reset at the start of every step.
__global__ void k_batch_gate( cudaGraphConditionalHandle h, int arm, int k, int *__restrict__ rec,
                              const int *__restrict__ flags, int nsp, int max_species )
{
    if( k == 0 ) {
        rec[0] = 0;
        rec[1] = 0;
        for( int i = 0; i < max_species; i++ ) rec[3 + i] = 0;
    } else if( !rec[0] && k - 1 < rec[2] ) {
        rec[1] = k;
        bool stop = flags[0] != 0;
        for( int i = 0; i < nsp; i++ ) {
            rec[3 + i] += flags[1 + max_species + i];
            stop = stop || flags[1 + i] > 0;
        }
        for( int i = 0; i < 1 + 2 * max_species; i++ ) rec[3 + max_species + i] = flags[i];
        if( stop ) rec[0] = 1;
    }
    if( arm ) cudaGraphSetConditional( h, ( !rec[0] && k < rec[2] ) ? 1u : 0u );
}

template <class T>
__global__ void k_fill( int64_t n, T *__restrict__ a, T v )
{
    const int64_t i = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x;
    if( i < n ) a[i] = v;
}

template <class Src, class Dst>
__global__ void k_convert( int64_t n, const Src *__restrict__ s, Dst *__restrict__ d )
{
    const int64_t i = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x;
    if( i < n ) d[i] = ( Dst )s[i];
}

__host__ __device__ inline size_t packed_header_bytes( int nt ) { return ( 8 + 4 * ( size_t )nt + 255 ) & ~( size_t )255; }

// Packed state: the particles of every tile back to back (tile order), plane by plane,
// behind the per-tile counts; pack reads the segments, unpack writes them back into the
// current layout (a tile's count must fit its segment).
template <bool MIXED>
__device__ __forceinline__ void packed_planes( const PBuf<MIXED> &, int ndim, int64_t n, char *base, PBuf<MIXED> &pk )
{
    using PT = typename std::conditional<MIXED, float, double>::type;
    char *q = base;
    if constexpr( MIXED ) {
        pk.key = reinterpret_cast<unsigned *>( q );
        q += 4 * n;
        for( int d = 0; d < 3; d++ ) {
            pk.d[d] = d < ndim ? reinterpret_cast<float *>( q ) : nullptr;
            if( d < ndim ) q += 4 * n;
        }
    } else {
        for( int d = 0; d < 3; d++ ) {
            pk.x[d] = d < ndim ? reinterpret_cast<double *>( q ) : nullptr;
            if( d < ndim ) q += 8 * n;
        }
    }
    for( int c = 0; c < 3; c++ ) {
        pk.p[c] = reinterpret_cast<PT *>( q );
        q += sizeof( PT ) * n;
    }
    pk.w = reinterpret_cast<PT *>( q );
    pk.tau = nullptr;
}

template <bool MIXED, bool PACK>
__global__ void k_pack( int ndim, int nt, const int64_t *__restrict__ seg_start, const int *__restrict__ cap,
                        int *__restrict__ count, const int64_t *__restrict__ off, PBuf<MIXED> b, int64_t n,
                        char *__restrict__ packed, int *__restrict__ status, int t0 )
{
    const int t = blockIdx.x + t0;
    if( t >= nt ) return;
    int *counts = reinterpret_cast<int *>( packed + 8 ); // behind the particle count (int64)
    PBuf<MIXED> pk;
    packed_planes<MIXED>( b, ndim, n, packed + packed_header_bytes( nt ), pk );
    b.tau = nullptr; // the optical depth stays in place
    int c;
    if constexpr( PACK ) {
        c = count[t];
        if( threadIdx.x == 0 ) counts[t] = c;
    } else {
        c = counts[t];
        if( c > cap[t] || c < 0 ) {
            if( threadIdx.x == 0 ) atomicCAS( status, 0, SG_ERR_ARG );
            return;
        }
        if( threadIdx.x == 0 ) count[t] = c;
    }
    for( int i = threadIdx.x; i < c; i += blockDim.x ) {
        if constexpr( PACK ) copy_particle<MIXED>( b, seg_start[t] + i, pk, off[t] + i, ndim );
        else copy_particle<MIXED>( pk, off[t] + i, b, seg_start[t] + i, ndim );
    }
}

// First and end packed particle of tiles [q0, q1) into pinned host memory. A store from
// the SMs, not a copy: a copy would queue on the copy engine behind the bulk copies out.
__global__ void k_store_bounds( const int64_t *__restrict__ off, int q0, int q1, int nt, int64_t n,
                                volatile int64_t *host )
{
    host[0] = off[q0];
    host[1] = q1 < nt ? off[q1] : n;
    __threadfence_system();
}

// Back to absolute FP64 positions (tile-sorted order) for output.
template <int DIM, bool MIXED>
__global__ void k_export( GridInfo g, int nt, const int64_t *__restrict__ seg_start, const int *__restrict__ count,
                          const int64_t *__restrict__ out_off, PBuf<MIXED> b, int64_t ntot, double *__restrict__ pos,
                          double *__restrict__ mom, double *__restrict__ wgt )
{
    const int t = blockIdx.x;
    if( t >= nt ) return;
    const int n = count[t];
    for( int i = threadIdx.x; i < n; i += blockDim.x ) {
        const int64_t src = seg_start[t] + i, o = out_off[t] + i;
        if constexpr( MIXED ) {
            int node[3];
            unpack_key( DIM, b.key[src], node[0], node[1], node[2] );
            for( int d = 0; d < DIM; d++ ) {
                double x = ( ( double )node[d] + ( double )b.d[d][src] ) * g.dx[d];
                if( x < 0.0 ) x += g.L[d];
                if( x >= g.L[d] ) x -= g.L[d];
                pos[d * ntot + o] = x;
            }
        } else {
            for( int d = 0; d < DIM; d++ ) pos[d * ntot + o] = b.x[d][src];
        }
        mom[o] = b.p[0][src];
        mom[ntot + o] = b.p[1][src];
        mom[2 * ntot + o] = b.p[2][src];
        wgt[o] = b.w[src];
    }
}

} // namespace
} // namespace sg

// ==============================================================================
// Host side: the sg_sim object.
// ==============================================================================
namespace sg {
namespace {

struct SpeciesState {
    double mass = 1.0, charge = -1.0;
    int pusher = 0;
    int64_t npart = 0;
    int64_t capacity = 0;
    void *mem[2] = { nullptr, nullptr };
    PBuf<false> bd[2]{};
    PBuf<true> bm[2]{};
    int cur = 0;
    int64_t *seg_start = nullptr;
    int *cap = nullptr;
    int *count[2] = { nullptr, nullptr };
    int64_t ovf_capacity = 0;
    void *ovf_mem = nullptr;
    PBuf<false> od{};
    PBuf<true> om{};
    int *ovf_tile = nullptr;
    int max_cap = 0; // largest tile segment of the current layout
    std::vector<int> h_cap;    // host copy of cap (the current layout's segment capacities)
    int *order = nullptr;      // tiles by decreasing capacity: the persistent kernel's queue order
    bool radiates = false;     // carries an optical-depth plane (Monte-Carlo radiation)
    void *tau_mem[2] = { nullptr, nullptr };
    void *ovf_tau = nullptr;
    const sg_rad_tables *rad_tables = nullptr; // its radiation tables and network (not owned)
    const sg_mlp *rad_mlp = nullptr;
    uint32_t rad_seed = 0;
    double *d_rad = nullptr;   // device tallies: radiated energy, emissions (as unsigned long long)
    // its macro-photons (RadiationMonteCarlo.cpp:425-545 with a photon species): a device
    // store of ph_cap photons (FP64: x, y; px, py, pz; weight; chi; tau planes of ph_cap)
    // and the count of photons wanted so far (may pass ph_cap: those are not stored)
    double *ph_mem = nullptr;
    int64_t ph_cap = 0;
    unsigned long long *ph_count = nullptr;
    int ph_sampling = 1, ph_max_emissions = 1;
    double ph_threshold = 2.0;
    double slack = 0.0;        // capacity slack of this species' layout (0: the configuration's)
    int64_t last_relayout = -1; // step of its last re-layout after a spill
    bool inject = false;       // fresh window cells are filled from this profile
    InjectParams inj{};        // its profile (x0, x1, n_moved set per call)
};

// Carves a particle SoA of `n` elements out of one allocation.
template <bool MIXED>
size_t pbuf_bytes( int ndim, int64_t n )
{
    return MIXED ? ( size_t )( 1 + ndim + 4 ) * 4 * ( size_t )n + 256 * 9 : ( size_t )( ndim + 4 ) * 8 * ( size_t )n + 256 * 9;
}

inline char *align256( char *p ) { return reinterpret_cast<char *>( ( reinterpret_cast<uintptr_t>( p ) + 255 ) & ~uintptr_t( 255 ) ); }

void carve( void *mem, int ndim, int64_t n, PBuf<false> &b )
{
    char *p = align256( static_cast<char *>( mem ) );
    for( int d = 0; d < 3; d++ ) {
        b.x[d] = d < ndim ? reinterpret_cast<double *>( p ) : nullptr;
        if( d < ndim ) p = align256( p + 8 * n );
    }
    for( int d = 0; d < 3; d++ ) { b.p[d] = reinterpret_cast<double *>( p ); p = align256( p + 8 * n ); }
    b.w = reinterpret_cast<double *>( p );
    b.tau = nullptr;
}

void carve( void *mem, int ndim, int64_t n, PBuf<true> &b )
{
    char *p = align256( static_cast<char *>( mem ) );
    b.key = reinterpret_cast<unsigned *>( p );
    p = align256( p + 4 * n );
    for( int d = 0; d < 3; d++ ) {
        b.d[d] = d < ndim ? reinterpret_cast<float *>( p ) : nullptr;
        if( d < ndim ) p = align256( p + 4 * n );
    }
    for( int d = 0; d < 3; d++ ) { b.p[d] = reinterpret_cast<float *>( p ); p = align256( p + 4 * n ); }
    b.w = reinterpret_cast<float *>( p );
    b.tau = nullptr;
}

} // namespace
} // namespace sg

using namespace sg;

struct sg_sim {
    sg_sim_config cfg{};
    GridInfo g{};
    bool mixed = false;
    size_t esz = 8;
    void *fmem = nullptr;
    void *fptr[12] = {};
    void *ecomp[3] = {}; // mixed form: compensation words of Ex, Ey, Ez
    int64_t fsize[12] = {};
    int fshape[12][3] = {};
    std::vector<SpeciesState> sp;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    bool tile_queue = false;  // particle kernel as a persistent grid over a tile queue
    int *d_queue = nullptr;   // its item counter
    bool tma = false;         // field tile staged by TMA (3D mixed, 4x4x4 tiles)
    float *tma_pad[6] = {};   // E, B_m with rows padded to a multiple of 4 values
    bool pad_dirty = true;    // E or B_m changed outside the field kernels (which keep the copies)
    int tma_nz4[6] = {};      // their padded row lengths
    TmaFields tma_maps{};     // tensor maps over them
    int *d_flags = nullptr; // [0] status, [1 + s] spill count of species s, [1 + max_species + s] removed
    int *h_flags = nullptr; // pinned copy
    int max_species = 16;
    int64_t *scan_scratch = nullptr;
    int64_t *tmp_start = nullptr;
    int *tmp_cap = nullptr;
    int *fill = nullptr;
    double *d_red = nullptr;
    cudaGraphExec_t graph[2] = { nullptr, nullptr };
    int graph_parity = -1; // parity of species 0 that graph[0] starts from
    // batched steps: BATCH_STEPS steps in one graph, each behind a conditional node that a
    // gate kernel arms while no earlier step of the batch spilled or failed, so that the
    // host waits for the device once per batch instead of once per step
    cudaGraphExec_t batch[2] = { nullptr, nullptr };
    int batch_parity = -1;        // parity of species 0 that batch[0] starts from
    bool batch_unsupported = false; // the runtime refused a batched graph: steps one by one
    int *d_batch = nullptr;       // gate record, layout at k_batch_gate
    int *h_batch = nullptr;       // its pinned copy (written by the graph's last node), then the step limit
    int64_t batches = 0, batched_steps = 0;
    cudaEvent_t ev[4] = { nullptr, nullptr, nullptr, nullptr }; // step start, particles start/end, step end
    float last_ms[3] = { 0, 0, 0 };
    int launches_per_step = 0;
    OpenBC obc{};                // Silver-Mueller coefficients and lasers (open axes)
    int64_t *d_step = nullptr;   // steps done (device), read by the boundary lasers
    int64_t relayouts = 0;       // segment re-layouts after a spill
    int64_t spilled = 0;         // particles that went through the spill list
    size_t smem_bytes = 0;
    int64_t hstep = 0;           // steps done (host copy)
    int64_t *d_rad_step = nullptr; // steps done (device), the radiation's random streams
    // moving window (SimWindow.cpp:93-96): moves `shift` cells when (time_dual - t_start) v > x_moved
    bool win_on = false;
    double win_t_start = 0.0, win_velocity = 0.0, win_x_moved = 0.0;
    int win_shift = 0;
    int64_t win_n_moved = 0;
    int64_t win_shifts = 0;
    void *win_scratch = nullptr;         // one field array
    int *slot_tile = nullptr;            // per particle slot: its tile after a shift (-1: removed)
    int64_t slot_cap = 0;
    unsigned long long *d_wcount = nullptr; // [0] removed, [1] created
    void *pack_mem = nullptr;    // staging of the packed state
    size_t pack_bytes = 0;
    cudaStream_t copy_stream = nullptr; // host-to-device copies of a streamed step
    cudaStream_t out_stream = nullptr;  // its device-to-host copies
    std::vector<cudaEvent_t> copy_ev;   // [0] staging free, [1] header copied, [2 + c] chunk c copied,
                                        // [2 + chunks + c] chunk c packed
    void *pack_out_mem = nullptr;       // staging of the packed state a streamed step writes
    size_t pack_out_cap = 0;
    int64_t *pack_off = nullptr;        // its per-tile offsets
    int64_t *h_chunk_end = nullptr;     // pinned: first and end packed particle of each range
    int64_t *d_chunk_end = nullptr;     // its device address
    float stream_ms[4] = { -1, -1, -1, -1 }; // last streamed step: copy in, particles, copy out, fields done
    // energy sums of the current state ([1] field, [2 + k] kinetic of species k), in pinned
    // memory; a streamed step computes them while its last ranges are copied out
    double *h_energy = nullptr;
    bool energy_valid = false;
    std::vector<int64_t> h_off; // streamed step: prefix of the packed tile counts (kept, not refaulted)
    size_t max_pitch = 0;       // the device's largest pitch for strided copies
};

namespace sg {
namespace {

// Bytes per element of field component c: J (9..11) is FP64 in both forms.
inline size_t felem( const sg_sim *S, int c ) { return c >= 9 ? 8 : S->esz; }

template <class T>
Fields<T> field_view( sg_sim *S )
{
    Fields<T> f;
    for( int c = 0; c < 3; c++ ) {
        f.E[c] = static_cast<T *>( S->fptr[c] );
        f.B[c] = static_cast<T *>( S->fptr[3 + c] );
        f.Bm[c] = static_cast<T *>( S->fptr[6 + c] );
        f.J[c] = static_cast<double *>( S->fptr[9 + c] );
        f.Ec[c] = static_cast<T *>( S->ecomp[c] );
    }
    return f;
}

// Where the field kernels write the padded copies of E and B_m (TMA staging only).
inline PadOut pad_out( const sg_sim *S )
{
    PadOut po{};
    if( S->tma )
        for( int c = 0; c < 6; c++ ) {
            po.p[c] = S->tma_pad[c];
            po.nz4[c] = S->tma_nz4[c];
        }
    return po;
}

// The padded copies from the arrays, where E or B_m changed outside the field kernels
// (a field set from the host, the Poisson solve, TMA staging switched on): each step's
// Ampere and Faraday kernels keep them current after that.
int pad_fields( sg_sim *S, cudaStream_t st )
{
    if( !S->tma || !S->pad_dirty ) return SG_OK;
    Fields<float> f = field_view<float>( S );
    for( int c = 0; c < 6; c++ ) {
        const float *src = c < 3 ? f.E[c] : f.Bm[c - 3];
        const int64_t rows = S->fsize[c] / S->fshape[c][2];
        k_pad_rows<<<( unsigned )std::min<int64_t>( ( rows * S->tma_nz4[c] + 255 ) / 256, 152 * 32 ), 256, 0, st>>>(
            src, S->tma_pad[c], rows, S->fshape[c][2], S->tma_nz4[c] );
        SG_LAUNCH_CHECK( "k_pad_rows" );
    }
    S->pad_dirty = false;
    return SG_OK;
}

// comp 0..2 E, 3..5 B, 6..8 B_m, 9..11 J -> staggering flags
inline int comp_stag( int comp, int d ) { return comp < 3 ? stag( comp, d ) : ( comp < 9 ? stag( 3 + ( comp % 3 ), d ) : stag( comp - 9, d ) ); }


template <int DIM, bool MIXED, int KIND>
int launch_particles( sg_sim *S, SpeciesState &s, cudaStream_t st, int t0, int t1 )
{
    using T = typename std::conditional<MIXED, float, double>::type;
    const int in = s.cur, out = 1 - s.cur;
    PBuf<MIXED> bin, bout, bov;
    if constexpr( MIXED ) { bin = s.bm[in]; bout = s.bm[out]; bov = s.om; }
    else { bin = s.bd[in]; bout = s.bd[out]; bov = s.od; }
    SpecParams sp;
    sp.charge = s.charge;
    sp.mass = s.mass;
    sp.qm_dts2 = s.charge / s.mass * S->g.dt * 0.5;
    double vol = 1.0;
    for( int d = 0; d < S->g.ndim; d++ ) vol *= S->g.dx[d];
    sp.cw = s.charge / vol;
    for( int d = 0; d < 3; d++ ) {
        sp.cr[d] = sp.cw * S->g.dx[d] / S->g.dt;
        sp.vs[d] = S->g.dt * S->g.dxi[d];
    }
    sp.f_qm_dts2 = ( float )sp.qm_dts2;
    sp.f_cw = ( float )sp.cw;
    for( int d = 0; d < 3; d++ ) {
        sp.f_cr[d] = ( float )sp.cr[d];
        sp.f_vs[d] = ( float )sp.vs[d];
    }
    sp.tile0 = t0;
    if( t1 <= t0 ) return SG_OK;
    // The mixed form deposits per cell (one tile = at most 64 cells in 3D, where two
    // thread groups split a cell's footprint, 128 in 2D).  Its particles go through
    // shared memory in chunks: the chunk is the largest segment when that fits the
    // budget of five blocks per SM, else the most that does.
    auto kern = k_step_particles<DIM, MIXED, KIND, false>;
    size_t smem = S->smem_bytes;
    int chunk = s.max_cap;
    if constexpr( MIXED ) {
        const int tc = S->g.T[0] * S->g.T[1] * ( DIM == 3 ? S->g.T[2] : 1 );
        const size_t j2 = cells_j2_bytes( tile_dims( S->g ) );
        const int fit = cells_chunk_fit( smem + j2, tc, true );
        chunk = std::max( 1, std::min( s.max_cap, fit & ~31 ) );
        if( tc <= ( DIM == 3 ? 64 : 128 ) && fit >= 128 ) {
            const GridInfo &g = S->g;
            int ft = 0;
            if( DIM == 3 ) ft = ( g.T[0] == 4 && g.T[1] == 4 && g.T[2] == 4 ) ? 1 : 0;
            else if( g.T[0] == 8 && g.T[1] == 8 ) ft = 1;
            else if( g.T[0] == 8 && g.T[1] == 16 ) ft = 2;
            else if( g.T[0] == 4 && g.T[1] == 4 ) ft = 3;
            if( ft ) {
                // the chunk is a compile-time constant of the kernel
                chunk = fixt_chunk( DIM, ft );
                if( chunk != ( fit & ~31 ) ) return set_error( SG_ERR_ARG, "per-cell chunk mismatch (%d, %d)", chunk, fit & ~31 );
            }
            kern = k_step_particles<DIM, MIXED, KIND, true>;
            if( ft == 1 ) kern = k_step_particles<DIM, MIXED, KIND, true, 1>;
            if constexpr( DIM == 2 ) {
                if( ft == 2 ) kern = k_step_particles<DIM, MIXED, KIND, true, 2>;
                if( ft == 3 ) kern = k_step_particles<DIM, MIXED, KIND, true, 3>;
            }
            smem += j2 + cells_smem_bytes( tc, chunk, true );
            if constexpr( DIM == 3 ) {
                if( S->tma && ft == 1 ) {
                    kern = k_step_particles<3, true, KIND, true, 1, true>;
                    chunk = tma_chunk();
                    smem = TMA_TILE_BYTES + cells_smem_bytes( tc, chunk, false );
                }
            }
        }
    }
    if( smem > 48 * 1024 ) SG_CUDA_TRY( cudaFuncSetAttribute( kern, cudaFuncAttributeMaxDynamicSharedMemorySize, ( int )smem ) );
    const int sidx = ( int )( &s - &S->sp[0] );
    sp.queue = nullptr;
    sp.order = nullptr;
    sp.nitems = t1 - t0;
    int grid = t1 - t0;
    if( S->tile_queue && t0 == 0 && t1 == S->g.ntiles && s.order ) {
        // persistent grid: as many CTAs as fit on the GPU at once, each taking tiles
        // from the queue, densest first
        int per_sm = 0, sms = 0, dev = 0;
        SG_CUDA_TRY( cudaGetDevice( &dev ) );
        SG_CUDA_TRY( cudaDeviceGetAttribute( &sms, cudaDevAttrMultiProcessorCount, dev ) );
        SG_CUDA_TRY( cudaOccupancyMaxActiveBlocksPerMultiprocessor( &per_sm, kern, 128, smem ) );
        grid = std::max( 1, std::min( t1 - t0, per_sm * sms ) );
        SG_CUDA_TRY( cudaMemsetAsync( S->d_queue, 0, sizeof( int ), st ) );
        sp.queue = S->d_queue;
        sp.order = s.order;
    }
    kern<<<grid, 128, smem, st>>>( S->g, field_view<T>( S ), sp, bin, bout, s.seg_start, s.cap, s.count[in],
                                          s.count[out], bov, s.ovf_tile, S->d_flags + 1 + sidx, ( int )s.ovf_capacity,
                                          S->d_flags, chunk, S->d_flags + 1 + S->max_species + sidx, S->tma_maps );
    SG_LAUNCH_CHECK( "k_step_particles" );
    return SG_OK;
}

template <int DIM, bool MIXED>
int launch_particles_kind( sg_sim *S, SpeciesState &s, cudaStream_t st, int t0, int t1 )
{
    if( s.pusher == 0 ) return launch_particles<DIM, MIXED, 0>( S, s, st, t0, t1 );
    if( s.pusher == 1 ) return launch_particles<DIM, MIXED, 1>( S, s, st, t0, t1 );
    return launch_particles<DIM, MIXED, 2>( S, s, st, t0, t1 );
}

// The particle step of species s over tiles [t0, t1) (all tiles by default).
int launch_particles_any( sg_sim *S, SpeciesState &s, cudaStream_t st, int t0 = 0, int t1 = -1 )
{
    if( t1 < 0 ) t1 = S->g.ntiles;
    if( S->g.ndim == 3 ) return S->mixed ? launch_particles_kind<3, true>( S, s, st, t0, t1 ) : launch_particles_kind<3, false>( S, s, st, t0, t1 );
    return S->mixed ? launch_particles_kind<2, true>( S, s, st, t0, t1 ) : launch_particles_kind<2, false>( S, s, st, t0, t1 );
}

template <int DIM, class T>
int launch_fields( sg_sim *S, cudaStream_t st, int &launches )
{
    Fields<T> f = field_view<T>( S );
    const GridInfo &g = S->g;
    for( int d = 0; d < DIM; d++ ) {
        if( g.open[d] ) continue; // ghost currents at an open boundary are not folded
        int64_t slab = 6;
        for( int k = 0; k < DIM; k++ )
            if( k != d ) slab *= g.np[k] + 1;
        dim3 grid( ( unsigned )std::min<int64_t>( ( slab + 255 ) / 256, 4096 ), 3 );
        k_fold<T><<<grid, 256, 0, st>>>( g, d, f );
        SG_LAUNCH_CHECK( "k_fold" );
        launches++;
    }
    const T dt = T( g.dt ), dtdx = T( g.dt / g.dx[0] ), dtdy = T( g.dt / g.dx[1] ), dtdz = T( DIM == 3 ? g.dt / g.dx[2] : 0.0 );
    const unsigned rows = DIM == 3 ? ( unsigned )( ( g.np[0] + 1 ) * ( g.np[1] + 1 ) ) : ( unsigned )( g.np[0] + 1 );
    const int tpb = DIM == 3 ? ( g.np[2] + 1 <= 128 ? 128 : 256 ) : 256;
    k_ampere_all<DIM, T><<<rows, tpb, 0, st>>>( g, f, dt, dtdx, dtdy, dtdz, pad_out( S ) );
    SG_LAUNCH_CHECK( "k_ampere_all" );
    if( DIM == 2 && ( g.open[0] || g.open[1] ) ) {
        const int64_t pts = ( int64_t )( g.np[0] + 1 ) * ( g.np[1] + 1 );
        const unsigned blocks = ( unsigned )( ( pts + 255 ) / 256 );
        k_faraday_open2d<T><<<blocks, 256, 0, st>>>( g, f, dtdx, dtdy );
        SG_LAUNCH_CHECK( "k_faraday_open2d" );
        const int nside = std::max( g.np[0], g.np[1] ) + 1;
        k_silver_mueller2d<T><<<dim3( ( nside + 127 ) / 128, 4 ), 128, 0, st>>>( g, f, S->obc, S->d_step );
        SG_LAUNCH_CHECK( "k_silver_mueller2d" );
        k_center_b2d<T><<<blocks, 256, 0, st>>>( g, f, S->d_step );
        SG_LAUNCH_CHECK( "k_center_b2d" );
        launches += 4;
        return SG_OK;
    }
    k_faraday_center<DIM, T><<<rows, tpb, 0, st>>>( g, f, dtdx, dtdy, dtdz, pad_out( S ) );
    SG_LAUNCH_CHECK( "k_faraday_center" );
    launches += 2;
    return SG_OK;
}

// The radiation pass over species s (2D mixed form) on its current buffer.
int launch_radiation( sg_sim *S, SpeciesState &s, cudaStream_t st )
{
    const GridInfo &g = S->g;
    ResidentRad r{};
    for( int d = 0; d < 2; d++ ) {
        r.N[d] = g.N[d];
        r.np[d] = g.np[d];
        r.T[d] = g.T[d];
        r.nt[d] = g.nt[d];
        r.dx[d] = g.dx[d];
        r.dxi[d] = g.dxi[d];
    }
    r.ntiles = g.ntiles;
    for( int c = 0; c < 3; c++ ) {
        r.E[c] = static_cast<const float *>( S->fptr[c] );
        r.Bm[c] = static_cast<const float *>( S->fptr[6 + c] );
    }
    const PBuf<true> &b = s.bm[s.cur];
    r.seg_start = s.seg_start;
    r.count = s.count[s.cur];
    r.nslots = s.capacity; // slots past the last segment find no particle
    r.key = b.key;
    r.d[0] = b.d[0];
    r.d[1] = b.d[1];
    for( int c = 0; c < 3; c++ ) r.p[c] = b.p[c];
    r.w = b.w;
    r.tau = b.tau;
    r.dt = g.dt;
    r.qm2 = s.charge / ( s.mass * s.mass );
    r.seed = s.rad_seed;
    r.step = S->d_rad_step;
    r.radiated = s.d_rad;
    r.emissions = reinterpret_cast<unsigned long long *>( s.d_rad + 1 );
    if( s.ph_mem ) {
        r.ph_sampling = s.ph_sampling;
        r.ph_max_emissions = s.ph_max_emissions;
        r.ph_threshold = s.ph_threshold;
        r.ph_cap = s.ph_cap;
        r.ph_count = s.ph_count;
        r.ph_pos = s.ph_mem;
        r.ph_mom = s.ph_mem + 2 * s.ph_cap;
        r.ph_w = s.ph_mem + 5 * s.ph_cap;
        r.ph_chi = s.ph_mem + 6 * s.ph_cap;
        r.ph_tau = s.ph_mem + 7 * s.ph_cap;
    }
    return launch_radiate_resident( s.rad_tables, s.rad_mlp, r, st );
}

// One species whose packed state streams in from host memory during the step. Its
// tiles go in ranges [ta[j], tb[j]), j in processing order; the copy stream has put
// range j's particles in the staging buffer when copy_ev[2 + j] fires.
//
// With `pack` set, the new state is packed range by range as well. Range j's output
// tiles are final once every tile within one tile of them has stepped, which is after
// the kernel of range pack_after[j]; and the packed offsets of range j depend only on
// tiles before it, which are final by then too.  Range j is then packed into the
// output staging, its first and last packed particle go to h_chunk_end[2j], [2j + 1],
// copy_ev[2 + nr + j] fires, and the host copies it out while later ranges still step.
struct StreamIn {
    int species = -1;
    int64_t n = 0;
    std::vector<int> ta, tb;
    bool pack = false;
    std::vector<int> pack_after;
};

// Unpacks the streamed species range by range and steps each range's tiles as soon as
// their particles are in, so the copies of later ranges overlap the particle kernel.
int stream_in_particles( sg_sim *S, SpeciesState &s, const StreamIn &in, cudaStream_t st, int &launches )
{
    const int nt = S->g.ntiles, nd = S->g.ndim, nr = ( int )in.ta.size();
    char *stg = static_cast<char *>( S->pack_mem );
    SG_CUDA_TRY( cudaStreamWaitEvent( st, S->copy_ev[1], 0 ) );
    int r = exclusive_scan<int>( reinterpret_cast<const int *>( stg + 8 ), nt, S->tmp_start, S->scan_scratch, st );
    if( r ) return r;
    for( int j = 0; j < nr; j++ ) {
        const int t0 = in.ta[j], t1 = in.tb[j];
        if( t1 > t0 ) {
            SG_CUDA_TRY( cudaStreamWaitEvent( st, S->copy_ev[2 + j], 0 ) );
            // a tile over its segment raises SG_ERR_ARG in the step status and keeps its old, in-bounds count
            if( S->mixed ) k_pack<true, false><<<t1 - t0, 128, 0, st>>>( nd, nt, s.seg_start, s.cap, s.count[s.cur], S->tmp_start, s.bm[s.cur], in.n, stg, S->d_flags, t0 );
            else k_pack<false, false><<<t1 - t0, 128, 0, st>>>( nd, nt, s.seg_start, s.cap, s.count[s.cur], S->tmp_start, s.bd[s.cur], in.n, stg, S->d_flags, t0 );
            SG_LAUNCH_CHECK( "k_pack" );
            r = launch_particles_any( S, s, st, t0, t1 );
            if( r ) return r;
            launches += 2;
        }
        for( int q = 0; in.pack && q < nr; q++ ) {
            if( in.pack_after[q] != j ) continue;
            const int out = 1 - s.cur, q0 = in.ta[q], q1 = in.tb[q];
            char *ostg = static_cast<char *>( S->pack_out_mem );
            r = exclusive_scan<int>( s.count[out], nt, S->pack_off, S->scan_scratch, st );
            if( r ) return r;
            if( q1 > q0 ) {
                if( S->mixed ) k_pack<true, true><<<q1 - q0, 128, 0, st>>>( nd, nt, s.seg_start, s.cap, s.count[out], S->pack_off, s.bm[out], in.n, ostg, S->d_flags, q0 );
                else k_pack<false, true><<<q1 - q0, 128, 0, st>>>( nd, nt, s.seg_start, s.cap, s.count[out], S->pack_off, s.bd[out], in.n, ostg, S->d_flags, q0 );
                SG_LAUNCH_CHECK( "k_pack" );
                launches++;
                k_store_bounds<<<1, 1, 0, st>>>( S->pack_off, q0, q1, nt, in.n, S->d_chunk_end + 2 * q );
                SG_LAUNCH_CHECK( "k_store_bounds" );
            }
            SG_CUDA_TRY( cudaEventRecord( S->copy_ev[2 + nr + q], st ) );
        }
    }
    return SG_OK;
}

// Enqueues one full timestep on `st` (no host synchronisation).  batched: the step is
// captured into the body of a conditional node, which holds no event records, so the
// stage events and the flags' copy to the host are left out (the batch's gates read the
// flags on the device).
int enqueue_step( sg_sim *S, cudaStream_t st, const StreamIn *in = nullptr, bool batched = false )
{
    int launches = 0;
    // inside a capture the stage events become external event nodes; outside, plain records
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    SG_CUDA_TRY( cudaStreamIsCapturing( st, &cs ) );
    const unsigned evflags = cs == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault;
    if( !batched ) SG_CUDA_TRY( cudaEventRecordWithFlags( S->ev[3], st, evflags ) );
    for( int c = 9; c < 12; c++ ) SG_CUDA_TRY( cudaMemsetAsync( S->fptr[c], 0, S->fsize[c] * felem( S, c ), st ) );
    SG_CUDA_TRY( cudaMemsetAsync( S->d_flags, 0, ( 1 + 2 * S->max_species ) * sizeof( int ), st ) );
    for( auto &s : S->sp ) SG_CUDA_TRY( cudaMemsetAsync( s.count[1 - s.cur], 0, S->g.ntiles * sizeof( int ), st ) );
    if( !batched ) SG_CUDA_TRY( cudaEventRecordWithFlags( S->ev[0], st, evflags ) );
    // Monte-Carlo radiation of the radiating species, before their push (Species.cpp:583-640)
    bool radiated = false;
    for( auto &s : S->sp ) {
        if( !s.radiates ) continue;
        int r = launch_radiation( S, s, st );
        if( r ) return r;
        launches++;
        radiated = true;
    }
    if( radiated ) {
        k_bump_step<<<1, 1, 0, st>>>( S->d_rad_step );
        SG_LAUNCH_CHECK( "k_bump_step" );
        launches++;
    }
    // the photon species' own push, over every stored photon, those just created too
    for( auto &s : S->sp ) {
        if( !s.ph_mem ) continue;
        const GridInfo &g = S->g;
        k_push_resident_photons<<<152 * 4, 256, 0, st>>>( s.ph_cap, s.ph_count, g.dt, s.ph_mem, s.ph_mem + 2 * s.ph_cap,
                                                          g.N[0] * g.dx[0], g.N[1] * g.dx[1], g.open[0] ? 0 : 1,
                                                          g.open[1] ? 0 : 1 );
        SG_LAUNCH_CHECK( "k_push_resident_photons" );
        launches++;
    }
    for( auto &s : S->sp ) {
        if( in && &s == &S->sp[in->species] ) {
            int r = stream_in_particles( S, s, *in, st, launches );
            if( r ) return r;
            continue;
        }
        int r = launch_particles_any( S, s, st );
        if( r ) return r;
        launches++;
    }
    if( !batched ) SG_CUDA_TRY( cudaEventRecordWithFlags( S->ev[1], st, evflags ) );
    int r;
    if( S->g.ndim == 3 ) r = S->mixed ? launch_fields<3, float>( S, st, launches ) : launch_fields<3, double>( S, st, launches );
    else r = S->mixed ? launch_fields<2, float>( S, st, launches ) : launch_fields<2, double>( S, st, launches );
    if( r ) return r;
    if( batched ) return SG_OK;
    SG_CUDA_TRY( cudaEventRecordWithFlags( S->ev[2], st, evflags ) );
    SG_CUDA_TRY( cudaMemcpyAsync( S->h_flags, S->d_flags, ( 1 + 2 * S->max_species ) * sizeof( int ), cudaMemcpyDeviceToHost, st ) );
    S->launches_per_step = launches;
    return SG_OK;
}

// The persistent kernel's tile order for species s: tiles by decreasing segment
// capacity (about their particle counts), so the densest tiles start first and the
// short ones fill the end.  Recomputed whenever the layout changes.
int refresh_order( sg_sim *S, SpeciesState &s )
{
    if( !S->tile_queue ) return SG_OK;
    const int nt = S->g.ntiles;
    if( ( int )s.h_cap.size() != nt ) return SG_OK;
    std::vector<int> idx( nt );
    for( int t = 0; t < nt; t++ ) idx[t] = t;
    std::stable_sort( idx.begin(), idx.end(), [&]( int a, int b ) { return s.h_cap[a] > s.h_cap[b]; } );
    if( !s.order ) SG_CUDA_TRY( cudaMalloc( &s.order, nt * sizeof( int ) ) );
    SG_CUDA_TRY( cudaMemcpyAsync( s.order, idx.data(), nt * sizeof( int ), cudaMemcpyHostToDevice, S->stream ) );
    SG_CUDA_TRY( cudaStreamSynchronize( S->stream ) );
    return SG_OK;
}

void drop_graphs( sg_sim *S )
{
    for( int i = 0; i < 2; i++ ) {
        if( S->graph[i] ) cudaGraphExecDestroy( S->graph[i] );
        S->graph[i] = nullptr;
        if( S->batch[i] ) cudaGraphExecDestroy( S->batch[i] );
        S->batch[i] = nullptr;
    }
    S->graph_parity = -1;
    S->batch_parity = -1;
}

int capture( sg_sim *S, cudaGraphExec_t *out )
{
    cudaGraph_t graph = nullptr;
    SG_CUDA_TRY( cudaStreamBeginCapture( S->stream, cudaStreamCaptureModeThreadLocal ) );
    int r = enqueue_step( S, S->stream );
    cudaError_t e = cudaStreamEndCapture( S->stream, &graph );
    if( r ) {
        if( graph ) cudaGraphDestroy( graph );
        return r;
    }
    if( e != cudaSuccess ) return cuda_fail( e, "cudaStreamEndCapture", __FILE__, __LINE__ );
    e = cudaGraphInstantiate( out, graph, 0 );
    cudaGraphDestroy( graph );
    if( e != cudaSuccess ) return cuda_fail( e, "cudaGraphInstantiate", __FILE__, __LINE__ );
    return SG_OK;
}

// Builds a graph of BATCH_STEPS steps from the species' current buffers: gate 0, step 0
// behind its conditional node, gate 1, step 1, ..., gate BATCH_STEPS (which accounts for
// the last step), then the record's copy to the host.  SG_OK with *out = null when the
// runtime refuses any part of it (the caller then steps one by one).
int build_batch( sg_sim *S, cudaGraphExec_t *out )
{
    *out = nullptr;
    cudaGraph_t g = nullptr;
    if( cudaGraphCreate( &g, 0 ) != cudaSuccess ) {
        cudaGetLastError();
        return SG_OK;
    }
    std::vector<int> cur0;
    for( auto &s : S->sp ) cur0.push_back( s.cur );
    const int nsp = ( int )S->sp.size();
    cudaGraphNode_t prev = nullptr;
    bool ok = true;
    int r = SG_OK;
    for( int k = 0; ok && r == SG_OK; k++ ) {
        const int arm = k < BATCH_STEPS ? 1 : 0;
        cudaGraphConditionalHandle h = 0;
        if( arm ) ok = cudaGraphConditionalHandleCreate( &h, g, 0, 0 ) == cudaSuccess;
        if( !ok ) break;
        void *args[] = { &h, ( void * )&arm, &k, &S->d_batch, &S->d_flags, ( void * )&nsp, &S->max_species };
        cudaKernelNodeParams kp{};
        kp.func = ( void * )k_batch_gate;
        kp.gridDim = dim3( 1 );
        kp.blockDim = dim3( 1 );
        kp.kernelParams = args;
        cudaGraphNode_t gate = nullptr;
        ok = cudaGraphAddKernelNode( &gate, g, prev ? &prev : nullptr, prev ? 1 : 0, &kp ) == cudaSuccess;
        prev = gate;
        if( !ok || !arm ) break;
        cudaGraphNodeParams cp{};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeIf;
        cp.conditional.size = 1;
        cudaGraphNode_t cn = nullptr;
        ok = cudaGraphAddNode( &cn, g, &prev, nullptr, 1, &cp ) == cudaSuccess;
        if( !ok ) break;
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        ok = cudaStreamBeginCaptureToGraph( S->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal ) ==
             cudaSuccess;
        if( !ok ) break;
        r = enqueue_step( S, S->stream, nullptr, true );
        ok = cudaStreamEndCapture( S->stream, &body ) == cudaSuccess;
        prev = cn;
        for( auto &s : S->sp ) s.cur = 1 - s.cur;
    }
    for( size_t i = 0; i < S->sp.size(); i++ ) S->sp[i].cur = cur0[i];
    cudaGraphNode_t cpy = nullptr;
    if( ok && r == SG_OK )
        ok = cudaGraphAddMemcpyNode1D( &cpy, g, &prev, 1, S->h_batch, S->d_batch,
                                       batch_record_ints( S->max_species ) * sizeof( int ), cudaMemcpyDeviceToHost ) ==
             cudaSuccess;
    if( ok && r == SG_OK ) ok = cudaGraphInstantiate( out, g, 0 ) == cudaSuccess;
    cudaGraphDestroy( g );
    if( !ok || r != SG_OK ) {
        if( *out ) cudaGraphExecDestroy( *out );
        *out = nullptr;
        cudaGetLastError(); // a refused batched graph leaves no error behind
    }
    return r;
}

// Optical-depth planes of a radiating species for both buffers (the old ones are
// left to the caller, who may still be reading them).
int alloc_tau( sg_sim *S, SpeciesState &s, int64_t capacity )
{
    for( int b = 0; b < 2; b++ ) {
        void *m = nullptr;
        if( cudaMalloc( &m, ( size_t )std::max<int64_t>( capacity, 1 ) * S->esz ) != cudaSuccess )
            return set_error( SG_ERR_NOMEM, "cannot allocate the optical-depth plane" );
        s.tau_mem[b] = m;
        if( S->mixed ) s.bm[b].tau = static_cast<float *>( m );
        else s.bd[b].tau = static_cast<double *>( m );
    }
    return SG_OK;
}

int alloc_species_buffers( sg_sim *S, SpeciesState &s, int64_t capacity )
{
    const int nd = S->g.ndim;
    const size_t bytes = S->mixed ? pbuf_bytes<true>( nd, capacity ) : pbuf_bytes<false>( nd, capacity );
    for( int b = 0; b < 2; b++ ) {
        void *m = nullptr;
        cudaError_t e = cudaMalloc( &m, bytes );
        if( e != cudaSuccess ) return set_error( SG_ERR_NOMEM, "cannot allocate %zu bytes of particle buffer", bytes );
        s.mem[b] = m;
        if( S->mixed ) carve( m, nd, capacity, s.bm[b] );
        else carve( m, nd, capacity, s.bd[b] );
    }
    s.capacity = capacity;
    if( s.radiates ) return alloc_tau( S, s, capacity );
    return SG_OK;
}

// New segment layout from counts: cap, seg_start into (new_cap, new_start); returns the total.
int layout_from_counts( sg_sim *S, const int *count, int *new_cap, int64_t *new_start, int64_t *total, int *max_cap,
                        std::vector<int> &caps, double slack_override = 0.0 )
{
    const int nt = S->g.ntiles;
    const float slack = ( float )( slack_override > 0.0 ? slack_override
                                                        : ( S->cfg.capacity_slack > 0.0 ? S->cfg.capacity_slack : 0.25 ) );
    // room beyond the slack fraction: 16 particles at the default slack of 0.25, less when the slack is smaller
    const int min_extra = ( int )std::ceil( 16.0 * std::min( 1.0, slack / 0.25 ) );
    k_caps<<<grid_for( nt, 256 ), 256, 0, S->stream>>>( S->g, count, new_cap, slack, min_extra );
    SG_LAUNCH_CHECK( "k_caps" );
    int r = exclusive_scan<int>( new_cap, nt, new_start, S->scan_scratch, S->stream );
    if( r ) return r;
    int64_t last_start = 0;
    int last_cap = 0;
    SG_CUDA_TRY( cudaMemcpyAsync( &last_start, new_start + nt - 1, sizeof( int64_t ), cudaMemcpyDeviceToHost, S->stream ) );
    SG_CUDA_TRY( cudaMemcpyAsync( &last_cap, new_cap + nt - 1, sizeof( int ), cudaMemcpyDeviceToHost, S->stream ) );
    caps.assign( nt, 0 );
    SG_CUDA_TRY( cudaMemcpyAsync( caps.data(), new_cap, nt * sizeof( int ), cudaMemcpyDeviceToHost, S->stream ) );
    SG_CUDA_TRY( cudaStreamSynchronize( S->stream ) );
    *total = last_start + last_cap;
    *max_cap = 0;
    for( int t = 0; t < nt; t++ ) *max_cap = std::max( *max_cap, caps[t] );
    return SG_OK;
}

template <bool MIXED>
int place_staged( sg_sim *S, SpeciesState &s, int64_t n, PBuf<MIXED> st, const int *st_tile, int dst_buf )
{
    if( n == 0 ) return SG_OK;
    PBuf<MIXED> dst;
    if constexpr( MIXED ) dst = s.bm[dst_buf];
    else dst = s.bd[dst_buf];
    k_place<MIXED><<<grid_for( n, 256 ), 256, 0, S->stream>>>( S->g.ndim, n, st, st_tile, s.seg_start, S->fill, dst );
    SG_LAUNCH_CHECK( "k_place" );
    return SG_OK;
}

// The per-cell chunk launch_particles passes for a largest segment of max_cap (0 for
// the FP64 form, whose kernel does not use it).  A new layout that keeps it, the
// segment tables and the buffers keeps the captured graphs valid.
template <int DIM>
int launch_chunk_dim( const sg_sim *S, int max_cap )
{
    if( !S->mixed ) return 0;
    const GridInfo &g = S->g;
    const int tc = g.T[0] * g.T[1] * ( DIM == 3 ? g.T[2] : 1 );
    const int fit = cells_chunk_fit( S->smem_bytes + cells_j2_bytes( tile_dims( g ) ), tc, true );
    int chunk = std::max( 1, std::min( max_cap, fit & ~31 ) );
    if( tc <= ( DIM == 3 ? 64 : 128 ) && fit >= 128 ) {
        int ft = 0;
        if( DIM == 3 ) ft = ( g.T[0] == 4 && g.T[1] == 4 && g.T[2] == 4 ) ? 1 : 0;
        else if( g.T[0] == 8 && g.T[1] == 8 ) ft = 1;
        else if( g.T[0] == 8 && g.T[1] == 16 ) ft = 2;
        else if( g.T[0] == 4 && g.T[1] == 4 ) ft = 3;
        if( ft ) chunk = fixt_chunk( DIM, ft );
    }
    return chunk;
}

int launch_chunk( const sg_sim *S, int max_cap )
{
    return S->g.ndim == 3 ? launch_chunk_dim<3>( S, max_cap ) : launch_chunk_dim<2>( S, max_cap );
}

// Steps within which a second spill doubles a species' capacity slack.
constexpr int64_t RELAYOUT_WINDOW = 64;

// Re-lays species s out after a spill: counts come from the step just done.
int relayout( sg_sim *S, SpeciesState &s, int nspill )
{
    const int nt = S->g.ntiles;
    int64_t total = 0;
    int new_max_cap = 0;
    // a species that spills again soon after its last re-layout gets twice the room per
    // tile (up to 2x its count): its density moves faster than the slack absorbs
    const double base = S->cfg.capacity_slack > 0.0 ? S->cfg.capacity_slack : 0.25;
    if( s.slack <= 0.0 ) s.slack = base;
    if( s.last_relayout >= 0 && S->hstep - s.last_relayout < RELAYOUT_WINDOW ) s.slack = std::min( 2.0, 2.0 * s.slack );
    s.last_relayout = S->hstep;
    std::vector<int> new_caps;
    int r = layout_from_counts( S, s.count[s.cur], S->tmp_cap, S->tmp_start, &total, &new_max_cap, new_caps, s.slack );
    if( r ) return r;
    // destination: the idle buffer, or fresh buffers when the layout no longer fits
    void *old_mem[2] = { s.mem[0], s.mem[1] }, *old_tau[2] = { s.tau_mem[0], s.tau_mem[1] };
    PBuf<false> old_bd = s.bd[s.cur];
    PBuf<true> old_bm = s.bm[s.cur];
    int dst_buf = 1 - s.cur;
    bool realloc = total > s.capacity;
    if( realloc ) {
        r = alloc_species_buffers( S, s, total + total / 8 );
        if( r ) return r;
        dst_buf = s.cur;
    }
    if( S->mixed )
        k_relayout_tiles<true><<<nt, 128, 0, S->stream>>>( S->g.ndim, nt, s.seg_start, s.cap, s.count[s.cur], old_bm, S->tmp_start, s.bm[dst_buf], S->fill );
    else
        k_relayout_tiles<false><<<nt, 128, 0, S->stream>>>( S->g.ndim, nt, s.seg_start, s.cap, s.count[s.cur], old_bd, S->tmp_start, s.bd[dst_buf], S->fill );
    SG_LAUNCH_CHECK( "k_relayout_tiles" );
    // new layout becomes current (copied into the same tables, which the graphs hold)
    const int old_chunk = launch_chunk( S, s.max_cap );
    SG_CUDA_TRY( cudaMemcpyAsync( s.seg_start, S->tmp_start, nt * sizeof( int64_t ), cudaMemcpyDeviceToDevice, S->stream ) );
    SG_CUDA_TRY( cudaMemcpyAsync( s.cap, S->tmp_cap, nt * sizeof( int ), cudaMemcpyDeviceToDevice, S->stream ) );
    s.max_cap = new_max_cap;
    s.h_cap.swap( new_caps );
    if( int ro = refresh_order( S, s ) ) return ro;
    if( S->mixed ) r = place_staged<true>( S, s, nspill, s.om, s.ovf_tile, dst_buf );
    else r = place_staged<false>( S, s, nspill, s.od, s.ovf_tile, dst_buf );
    if( r ) return r;
    SG_CUDA_TRY( cudaMemcpyAsync( s.count[dst_buf], s.count[s.cur], nt * sizeof( int ), cudaMemcpyDeviceToDevice, S->stream ) );
    SG_CUDA_TRY( cudaStreamSynchronize( S->stream ) );
    if( realloc ) {
        release( old_mem[0] );
        release( old_mem[1] );
        if( s.radiates ) {
            release( old_tau[0] );
            release( old_tau[1] );
        }
    }
    s.cur = dst_buf;
    // the graphs hold one buffer parity for all species together: a re-layout of one
    // species among several breaks it
    if( realloc || S->sp.size() > 1 || launch_chunk( S, s.max_cap ) != old_chunk ) drop_graphs( S );
    return SG_OK;
}

// Moves species s `shift` cells towards xmin (0: none), drops what left through
// xmin, adds the particles of its profile in window cells [x0, x1) (x0 == x1:
// none) and lays the species out anew.  Synchronises the stream.
int rebuild_species( sg_sim *S, SpeciesState &s, int shift, int x0, int x1 )
{
    const int nt = S->g.ntiles, nd = S->g.ndim;
    cudaStream_t st = S->stream;
    if( S->slot_cap < s.capacity ) {
        release( S->slot_tile );
        S->slot_tile = nullptr;
        S->slot_cap = 0;
        SG_CUDA_TRY( cudaMalloc( &S->slot_tile, s.capacity * sizeof( int ) ) );
        S->slot_cap = s.capacity;
    }
    if( !S->d_wcount ) SG_CUDA_TRY( cudaMalloc( &S->d_wcount, 2 * sizeof( unsigned long long ) ) );
    int *newcount = s.count[1 - s.cur];
    SG_CUDA_TRY( cudaMemsetAsync( newcount, 0, nt * sizeof( int ), st ) );
    SG_CUDA_TRY( cudaMemsetAsync( S->d_wcount, 0, 2 * sizeof( unsigned long long ), st ) );
    const int *cnt = s.count[s.cur];
    if( S->mixed ) {
        if( nd == 3 ) k_window_particles<3, true><<<nt, 128, 0, st>>>( S->g, s.seg_start, cnt, s.bm[s.cur], shift, S->slot_tile, newcount, S->d_wcount );
        else k_window_particles<2, true><<<nt, 128, 0, st>>>( S->g, s.seg_start, cnt, s.bm[s.cur], shift, S->slot_tile, newcount, S->d_wcount );
    } else {
        if( nd == 3 ) k_window_particles<3, false><<<nt, 128, 0, st>>>( S->g, s.seg_start, cnt, s.bd[s.cur], shift, S->slot_tile, newcount, S->d_wcount );
        else k_window_particles<2, false><<<nt, 128, 0, st>>>( S->g, s.seg_start, cnt, s.bd[s.cur], shift, S->slot_tile, newcount, S->d_wcount );
    }
    SG_LAUNCH_CHECK( "k_window_particles" );
    const bool inject = s.inject && x1 > x0;
    InjectParams ip = s.inj;
    ip.x0 = x0;
    ip.x1 = x1;
    ip.n_moved = ( long long )S->win_n_moved;
    const int64_t ncell = inject ? ( int64_t )( x1 - x0 ) * S->g.N[1] * ( nd == 3 ? S->g.N[2] : 1 ) : 0;
    const unsigned iblocks = ( unsigned )( ( ncell + 127 ) / 128 );
    auto launch_inject = [&]( int pass, PBuf<true> dm, PBuf<false> dd ) {
        if( S->mixed ) {
            if( nd == 3 ) k_inject<3, true><<<iblocks, 128, 0, st>>>( S->g, ip, pass, newcount, S->d_wcount + 1, S->tmp_start, S->fill, dm );
            else k_inject<2, true><<<iblocks, 128, 0, st>>>( S->g, ip, pass, newcount, S->d_wcount + 1, S->tmp_start, S->fill, dm );
        } else {
            if( nd == 3 ) k_inject<3, false><<<iblocks, 128, 0, st>>>( S->g, ip, pass, newcount, S->d_wcount + 1, S->tmp_start, S->fill, dd );
            else k_inject<2, false><<<iblocks, 128, 0, st>>>( S->g, ip, pass, newcount, S->d_wcount + 1, S->tmp_start, S->fill, dd );
        }
    };
    if( inject ) {
        launch_inject( 0, s.bm[s.cur], s.bd[s.cur] );
        SG_LAUNCH_CHECK( "k_inject (count)" );
    }
    int64_t total = 0;
    int new_max_cap = 0;
    std::vector<int> new_caps;
    int r = layout_from_counts( S, newcount, S->tmp_cap, S->tmp_start, &total, &new_max_cap, new_caps, s.slack ); // synchronises
    if( r ) return r;
    unsigned long long wc[2] = { 0, 0 };
    SG_CUDA_TRY( cudaMemcpyAsync( wc, S->d_wcount, sizeof( wc ), cudaMemcpyDeviceToHost, st ) );
    SG_CUDA_TRY( cudaStreamSynchronize( st ) );
    void *old_mem[2] = { s.mem[0], s.mem[1] }, *old_tau[2] = { s.tau_mem[0], s.tau_mem[1] };
    const PBuf<false> old_bd = s.bd[s.cur];
    const PBuf<true> old_bm = s.bm[s.cur];
    int dst = 1 - s.cur;
    const bool realloc = total > s.capacity;
    if( realloc ) {
        r = alloc_species_buffers( S, s, total + total / 8 );
        if( r ) return r;
        dst = s.cur;
    }
    SG_CUDA_TRY( cudaMemsetAsync( S->fill, 0, nt * sizeof( int ), st ) );
    if( S->mixed ) k_window_place<true><<<nt, 128, 0, st>>>( nd, s.seg_start, cnt, old_bm, S->slot_tile, S->tmp_start, S->fill, s.bm[dst] );
    else k_window_place<false><<<nt, 128, 0, st>>>( nd, s.seg_start, cnt, old_bd, S->slot_tile, S->tmp_start, S->fill, s.bd[dst] );
    SG_LAUNCH_CHECK( "k_window_place" );
    if( inject ) {
        launch_inject( 1, s.bm[dst], s.bd[dst] );
        SG_LAUNCH_CHECK( "k_inject (place)" );
    }
    SG_CUDA_TRY( cudaMemcpyAsync( s.count[dst], S->fill, nt * sizeof( int ), cudaMemcpyDeviceToDevice, st ) );
    // new layout into the same tables, which the graphs hold
    SG_CUDA_TRY( cudaMemcpyAsync( s.seg_start, S->tmp_start, nt * sizeof( int64_t ), cudaMemcpyDeviceToDevice, st ) );
    SG_CUDA_TRY( cudaMemcpyAsync( s.cap, S->tmp_cap, nt * sizeof( int ), cudaMemcpyDeviceToDevice, st ) );
    SG_CUDA_TRY( cudaStreamSynchronize( st ) );
    const int old_chunk = launch_chunk( S, s.max_cap );
    s.max_cap = new_max_cap;
    s.h_cap.swap( new_caps );
    if( int ro = refresh_order( S, s ) ) return ro;
    s.cur = dst;
    s.npart += ( int64_t )wc[1] - ( int64_t )wc[0];
    if( realloc ) {
        release( old_mem[0] );
        release( old_mem[1] );
        if( s.radiates ) {
            release( old_tau[0] );
            release( old_tau[1] );
        }
    }
    if( realloc || launch_chunk( S, s.max_cap ) != old_chunk ) drop_graphs( S );
    return SG_OK;
}

// The window's shift at the end of a step (SimWindow::shift): fields move
// `shift` cells towards xmin with zeros in the fresh cells, Silver-Mueller on
// xmin without laser (SimWindow.cpp:420-431), lasers off for good
// (laserDisabled, :138-145), particles follow and the fresh cells are filled.
int window_shift( sg_sim *S )
{
    S->pad_dirty = true; // the fields move
    const int P = S->win_shift;
    const GridInfo &g = S->g;
    cudaStream_t st = S->stream;
    std::vector<void *> arrays;
    std::vector<int> stag;
    for( int c = 0; c < 12; c++ ) {
        arrays.push_back( S->fptr[c] );
        stag.push_back( S->fshape[c][0] - g.np[0] );
    }
    for( int c = 0; c < 3; c++ )
        if( S->ecomp[c] ) {
            arrays.push_back( S->ecomp[c] );
            stag.push_back( S->fshape[c][0] - g.np[0] );
        }
    for( size_t a = 0; a < arrays.size(); a++ ) {
        const int c = a < 12 ? ( int )a : ( int )a - 12;
        const int64_t ex = S->fshape[c][0], plane = S->fsize[c] / ex;
        const int64_t keep = ( int64_t )g.N[0] - P + OS + stag[a];
        const int64_t n = S->fsize[c];
        const unsigned blocks = ( unsigned )std::min<int64_t>( ( n + 255 ) / 256, 152 * 16 );
        const size_t el = a < 12 ? felem( S, c ) : S->esz;
        if( el == 4 ) {
            k_window_shift_field<float><<<blocks, 256, 0, st>>>( static_cast<const float *>( arrays[a] ), static_cast<float *>( S->win_scratch ), ex, plane, keep, P );
        } else {
            k_window_shift_field<double><<<blocks, 256, 0, st>>>( static_cast<const double *>( arrays[a] ), static_cast<double *>( S->win_scratch ), ex, plane, keep, P );
        }
        SG_LAUNCH_CHECK( "k_window_shift_field" );
        SG_CUDA_TRY( cudaMemcpyAsync( arrays[a], S->win_scratch, n * el, cudaMemcpyDeviceToDevice, st ) );
    }
    const bool lasers_were_on = S->obc.nlaser > 0;
    S->obc.nlaser = 0;
    OpenBC xmin = S->obc;
    xmin.side_mask = 1;
    const int nside = std::max( g.np[0], g.np[1] ) + 1;
    if( S->mixed ) k_silver_mueller2d<float><<<dim3( ( nside + 127 ) / 128, 4 ), 128, 0, st>>>( g, field_view<float>( S ), xmin, S->d_step );
    else k_silver_mueller2d<double><<<dim3( ( nside + 127 ) / 128, 4 ), 128, 0, st>>>( g, field_view<double>( S ), xmin, S->d_step );
    SG_LAUNCH_CHECK( "k_silver_mueller2d" );
    S->win_n_moved += P;
    for( auto &s : S->sp ) {
        int r = rebuild_species( S, s, P, g.N[0] - P, g.N[0] );
        if( r ) return r;
    }
    SG_CUDA_TRY( cudaStreamSynchronize( st ) );
    S->win_shifts++;
    if( lasers_were_on ) drop_graphs( S ); // the boundary kernel holds the lasers by value
    return SG_OK;
}

int choose_tiles( sg_sim *S )
{
    GridInfo &g = S->g;
    for( int d = 0; d < 3; d++ ) {
        if( d >= g.ndim ) { g.T[d] = 1; g.nt[d] = 1; g.tshift[d] = 0; continue; }
        int t = S->cfg.tile[d];
        if( t <= 0 ) {
            const int pref = g.ndim == 3 ? 4 : 8;
            t = pref;
            while( t > 1 && g.N[d] % t ) t--;
        }
        if( g.N[d] % t ) return set_error( SG_ERR_ARG, "tile size %d does not divide %d cells in dimension %d", t, g.N[d], d );
        g.T[d] = t;
        // an open axis has N + 1 nodes (a particle in [L - dx/2, L) is nearest to node N): one more tile
        g.nt[d] = g.N[d] / t + g.open[d];
        g.tshift[d] = ( t & ( t - 1 ) ) == 0 ? __builtin_ctz( ( unsigned )t ) : -1;
    }
    g.ntiles = g.nt[0] * g.nt[1] * ( g.ndim == 3 ? g.nt[2] : 1 );
    const TileDims td = tile_dims( g );
    S->smem_bytes = ( size_t )( 6 * td.FX * td.FY * td.FZ + 3 * jtile_size( td ) ) * S->esz;
    if( S->smem_bytes > 200 * 1024 ) return set_error( SG_ERR_ARG, "tile too large for shared memory (%zu bytes)", S->smem_bytes );
    return SG_OK;
}

} // namespace
} // namespace sg

extern "C" {

int sg_sim_create( const sg_sim_config *cfg, sg_sim **out )
{
    SG_REQUIRE( cfg && out, "NULL argument" );
    SG_REQUIRE( cfg->ndim == 2 || cfg->ndim == 3, "ndim must be 2 or 3" );
    SG_REQUIRE( cfg->form == SG_FORM_FP64 || cfg->form == SG_FORM_MIXED, "unknown form %d", cfg->form );
    SG_REQUIRE( cfg->dt > 0.0, "dt must be positive" );
    for( int d = 0; d < cfg->ndim; d++ ) {
        SG_REQUIRE( cfg->n_cells[d] >= 8, "at least 8 cells per dimension are needed (dimension %d has %d)", d, cfg->n_cells[d] );
        SG_REQUIRE( cfg->cell_length[d] > 0.0, "cell_length[%d] must be positive", d );
        if( cfg->form == SG_FORM_MIXED )
            SG_REQUIRE( cfg->n_cells[d] + ( cfg->bc[d] == SG_BC_OPEN ) <= ( cfg->ndim == 3 ? ( d == 0 ? 2048 : 1024 ) : 65536 ),
                        "mixed form: too many cells in dimension %d", d );
        SG_REQUIRE( cfg->bc[d] == SG_BC_PERIODIC || cfg->bc[d] == SG_BC_OPEN, "unknown boundary %d in dimension %d", cfg->bc[d], d );
        SG_REQUIRE( cfg->bc[d] == SG_BC_PERIODIC || cfg->ndim == 2, "open boundaries are implemented in 2D" );
        SG_REQUIRE( cfg->dt < cfg->cell_length[d], "dt must be below every cell length (a particle may cross at most one cell per step)" );
    }
    sg_sim *S = new sg_sim();
    S->cfg = *cfg;
    S->mixed = cfg->form == SG_FORM_MIXED;
    S->esz = S->mixed ? 4 : 8;
    GridInfo &g = S->g;
    g.ndim = cfg->ndim;
    g.dt = cfg->dt;
    for( int d = 0; d < 3; d++ ) {
        g.open[d] = d < g.ndim && cfg->bc[d] == SG_BC_OPEN ? 1 : 0;
        g.N[d] = d < g.ndim ? cfg->n_cells[d] : 1;
        g.np[d] = d < g.ndim ? g.N[d] + 1 + 2 * OS : 1;
        g.dx[d] = d < g.ndim ? cfg->cell_length[d] : 1.0;
        g.dxi[d] = 1.0 / g.dx[d];
        g.L[d] = g.N[d] * g.dx[d];
    }
    int r = choose_tiles( S );
    if( r ) { delete S; return r; }
    S->obc.side_mask = 0xF;
    // Silver-Mueller coefficients (ElectroMagnBC2D_SM constructor, ElectroMagnBC2D_SM.cpp:18-66)
    // with the default incoming directions +x, -x, +y, -y (Params.cpp:476-493)
    for( int side = 0; side < 4 && g.ndim == 2; side++ ) {
        const int a0 = side / 2, a1 = a0 == 0 ? 1 : 0;
        const double sgn = ( double )( side % 2 ) * 2.0 - 1.0;
        const double k[2] = { a0 == 0 ? -sgn : 0.0, a0 == 1 ? -sgn : 0.0 };
        const double k0 = k[a0], k1 = k[a1];
        const double dt0 = g.dt / g.dx[a0], dt1 = g.dt / g.dx[a1];
        const double factor = 1.0 / ( k0 - sgn * dt0 );
        double *c = S->obc.coef[side];
        c[0] = 2.0 * factor;
        c[1] = -( k0 + sgn * dt0 ) * factor;
        c[2] = 4.0 * k0 * factor;
        c[3] = -( k1 + dt1 ) * factor;
        c[4] = -( k1 - dt1 ) * factor;
    }
    // fields
    size_t total = 0;
    for( int c = 0; c < 12; c++ ) {
        int64_t n = 1;
        for( int d = 0; d < 3; d++ ) {
            S->fshape[c][d] = ext( g, d, comp_stag( c, d ) );
            n *= S->fshape[c][d];
        }
        S->fsize[c] = n;
        total += ( ( n * felem( S, c ) + 255 ) / 256 ) * 256;
    }
    if( S->mixed )
        for( int c = 0; c < 3; c++ ) total += ( ( S->fsize[c] * S->esz + 255 ) / 256 ) * 256;
    cudaError_t e = cudaMalloc( &S->fmem, total );
    if( e != cudaSuccess ) { delete S; return set_error( SG_ERR_NOMEM, "cannot allocate %zu bytes of fields", total ); }
    cudaMemset( S->fmem, 0, total );
    char *p = static_cast<char *>( S->fmem );
    for( int c = 0; c < 12; c++ ) {
        S->fptr[c] = p;
        p += ( ( S->fsize[c] * felem( S, c ) + 255 ) / 256 ) * 256;
    }
    if( S->mixed )
        for( int c = 0; c < 3; c++ ) {
            S->ecomp[c] = p;
            p += ( ( S->fsize[c] * S->esz + 255 ) / 256 ) * 256;
        }
    const int nt = g.ntiles;
    e = cudaMalloc( &S->d_step, sizeof( int64_t ) );
    if( e == cudaSuccess ) e = cudaMemset( S->d_step, 0, sizeof( int64_t ) );
    if( e == cudaSuccess ) e = cudaMalloc( &S->d_flags, ( 1 + 2 * S->max_species ) * sizeof( int ) );
    if( e == cudaSuccess ) e = cudaMallocHost( &S->h_flags, ( 1 + 2 * S->max_species ) * sizeof( int ) );
    if( e == cudaSuccess ) e = cudaMalloc( &S->d_batch, batch_record_ints( S->max_species ) * sizeof( int ) );
    if( e == cudaSuccess ) e = cudaMallocHost( &S->h_batch, ( batch_record_ints( S->max_species ) + 1 ) * sizeof( int ) );
    if( e == cudaSuccess ) e = cudaMallocHost( &S->h_energy, 16 * sizeof( double ) );
    if( e == cudaSuccess ) e = cudaMalloc( &S->scan_scratch, scan_scratch_elems( nt ) * sizeof( int64_t ) );
    if( e == cudaSuccess ) e = cudaMalloc( &S->tmp_start, nt * sizeof( int64_t ) );
    if( e == cudaSuccess ) e = cudaMalloc( &S->tmp_cap, nt * sizeof( int ) );
    if( e == cudaSuccess ) e = cudaMalloc( &S->fill, nt * sizeof( int ) );
    if( e == cudaSuccess ) e = cudaMalloc( &S->d_red, 16 * sizeof( double ) );
    if( e == cudaSuccess ) e = cudaStreamCreateWithFlags( &S->stream, cudaStreamNonBlocking );
    for( int i = 0; i < 4 && e == cudaSuccess; i++ ) e = cudaEventCreate( &S->ev[i] );
    if( e != cudaSuccess ) {
        sg_sim_destroy( S );
        return cuda_fail( e, "sg_sim_create allocations", __FILE__, __LINE__ );
    }
    S->own_stream = true;
    // the 3D mixed form with 4x4x4 tiles on a periodic grid stages its field tile by TMA
    if( g.ndim == 3 && S->mixed && g.T[0] == 4 && g.T[1] == 4 && g.T[2] == 4 && !g.open[0] && !g.open[1] && !g.open[2] ) {
        const int r = sg_sim_set_tma_staging( S, 1 );
        if( r ) {
            sg_sim_destroy( S );
            return r;
        }
    }
    *out = S;
    return SG_OK;
}

int sg_sim_destroy( sg_sim *S )
{
    if( !S ) return SG_OK;
    if( S->stream ) cudaStreamSynchronize( S->stream );
    drop_graphs( S );
    for( auto &s : S->sp ) {
        release( s.mem[0] );
        release( s.mem[1] );
        release( s.seg_start );
        release( s.cap );
        release( s.order );
        release( s.count[0] );
        release( s.count[1] );
        release( s.ovf_mem );
        release( s.ovf_tile );
        release( s.tau_mem[0] );
        release( s.tau_mem[1] );
        release( s.ovf_tau );
        release( s.d_rad );
        release( s.ph_mem );
        release( s.ph_count );
    }
    release( S->d_rad_step );
    release( S->fmem );
    release( S->d_flags );
    release( S->d_queue );
    for( int c = 0; c < 6; c++ ) release( S->tma_pad[c] );
    release( S->d_step );
    if( S->h_flags ) cudaFreeHost( S->h_flags );
    release( S->d_batch );
    if( S->h_batch ) cudaFreeHost( S->h_batch );
    if( S->h_energy ) cudaFreeHost( S->h_energy );
    release( S->scan_scratch );
    release( S->tmp_start );
    release( S->tmp_cap );
    release( S->fill );
    release( S->d_red );
    release( S->win_scratch );
    release( S->pack_mem );
    release( S->slot_tile );
    release( S->d_wcount );
    for( int i = 0; i < 4; i++ )
        if( S->ev[i] ) cudaEventDestroy( S->ev[i] );
    for( cudaEvent_t e : S->copy_ev ) cudaEventDestroy( e );
    for( cudaStream_t x : { S->copy_stream, S->out_stream } )
        if( x ) {
            cudaStreamSynchronize( x );
            cudaStreamDestroy( x );
        }
    release( S->pack_out_mem );
    release( S->pack_off );
    if( S->h_chunk_end ) cudaFreeHost( S->h_chunk_end );
    if( S->own_stream && S->stream ) cudaStreamDestroy( S->stream );
    delete S;
    return SG_OK;
}

int sg_sim_set_tma_staging( sg_sim *S, int on )
{
    SG_REQUIRE( S, "NULL simulation" );
    SG_CUDA_TRY( cudaStreamSynchronize( S->stream ) );
    if( !on ) {
        S->tma = false;
        drop_graphs( S );
        return SG_OK;
    }
    const GridInfo &g = S->g;
    SG_REQUIRE( g.ndim == 3 && S->mixed && g.T[0] == 4 && g.T[1] == 4 && g.T[2] == 4,
                "TMA staging needs the 3D mixed form with 4x4x4 tiles" );
    SG_REQUIRE( !g.open[0] && !g.open[1] && !g.open[2], "TMA staging needs a periodic grid" );
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q{};
    SG_CUDA_TRY( cudaGetDriverEntryPointByVersion( "cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q ) );
    SG_REQUIRE( fn && q == cudaDriverEntryPointSuccess, "cuTensorMapEncodeTiled is not available" );
    auto encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>( fn );
    for( int c = 0; c < 6; c++ ) {
        const int field = c < 3 ? c : 6 + ( c - 3 ); // E, then B_m
        const int nx = S->fshape[field][0], ny = S->fshape[field][1], nz = S->fshape[field][2];
        S->tma_nz4[c] = ( nz + 3 ) & ~3;
        if( !S->tma_pad[c] ) SG_CUDA_TRY( cudaMalloc( &S->tma_pad[c], ( size_t )nx * ny * S->tma_nz4[c] * sizeof( float ) ) );
        const cuuint64_t dims[3] = { ( cuuint64_t )nz, ( cuuint64_t )ny, ( cuuint64_t )nx };
        const cuuint64_t strides[2] = { ( cuuint64_t )S->tma_nz4[c] * 4, ( cuuint64_t )S->tma_nz4[c] * 4 * ny };
        const cuuint32_t box[3] = { TMA_BOX_Z, TMA_BOX_Y, TMA_BOX_X }, estr[3] = { 1, 1, 1 };
        const CUresult r = encode( &S->tma_maps.m[c], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, S->tma_pad[c], dims, strides, box, estr,
                                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE );
        if( r != CUDA_SUCCESS ) return set_error( SG_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d) for field %d", ( int )r, field );
    }
    S->tma = true;
    S->pad_dirty = true;
    drop_graphs( S );
    return SG_OK;
}

int sg_sim_set_tile_queue( sg_sim *S, int on )
{
    SG_REQUIRE( S, "NULL simulation" );
    SG_CUDA_TRY( cudaStreamSynchronize( S->stream ) );
    S->tile_queue = on != 0;
    if( S->tile_queue && !S->d_queue ) SG_CUDA_TRY( cudaMalloc( &S->d_queue, sizeof( int ) ) );
    for( auto &s : S->sp ) {
        int r = refresh_order( S, s );
        if( r ) return r;
    }
    drop_graphs( S );
    return SG_OK;
}

int sg_sim_set_stream( sg_sim *S, sg_stream_t stream )
{
    SG_REQUIRE( S, "NULL simulation" );
    SG_CUDA_TRY( cudaStreamSynchronize( S->stream ) );
    if( S->own_stream ) cudaStreamDestroy( S->stream );
    S->stream = as_stream( stream );
    S->own_stream = false;
    drop_graphs( S );
    return SG_OK;
}

int sg_sim_add_species_device( sg_sim *S, double mass, double charge, int pusher, int64_t npart, const double *pos,
                               const double *mom, const double *weight, int *index )
{
    if( S ) S->energy_valid = false;
    SG_REQUIRE( S, "NULL simulation" );
    SG_REQUIRE( mass > 0.0, "mass must be positive" );
    SG_REQUIRE( pusher >= 0 && pusher <= 2, "pusher must be 0 (boris), 1 (vay) or 2 (higueracary)" );
    SG_REQUIRE( npart >= 0 && npart < ( int64_t )1 << 31, "npart out of range" );
    SG_REQUIRE( ( int )S->sp.size() < S->max_species, "too many species" );
    if( npart > 0 ) SG_REQUIRE( pos && mom && weight, "NULL particle array" );
    // the arrays may still be being written on another stream (the simulation's own
    // stream does not wait for the legacy default stream): let all device work end first
    SG_CUDA_TRY( cudaDeviceSynchronize() );
    const int nt = S->g.ntiles, nd = S->g.ndim;
    S->sp.emplace_back();
    SpeciesState &s = S->sp.back();
    s.mass = mass;
    s.charge = charge;
    s.pusher = pusher;
    s.npart = npart;
    cudaStream_t st = S->stream;
    SG_CUDA_TRY( cudaMalloc( &s.seg_start, nt * sizeof( int64_t ) ) );
    SG_CUDA_TRY( cudaMalloc( &s.cap, nt * sizeof( int ) ) );
    SG_CUDA_TRY( cudaMalloc( &s.count[0], nt * sizeof( int ) ) );
    SG_CUDA_TRY( cudaMalloc( &s.count[1], nt * sizeof( int ) ) );
    SG_CUDA_TRY( cudaMemsetAsync( s.count[0], 0, nt * sizeof( int ), st ) );
    SG_CUDA_TRY( cudaMemsetAsync( s.count[1], 0, nt * sizeof( int ), st ) );
    // spill list (also used as the staging area here)
    s.ovf_capacity = std::max<int64_t>( npart, std::max<int64_t>( 4096, npart / 16 ) );
    const size_t obytes = S->mixed ? pbuf_bytes<true>( nd, s.ovf_capacity ) : pbuf_bytes<false>( nd, s.ovf_capacity );
    SG_CUDA_TRY( cudaMalloc( &s.ovf_mem, obytes ) );
    SG_CUDA_TRY( cudaMalloc( &s.ovf_tile, s.ovf_capacity * sizeof( int ) ) );
    if( S->mixed ) carve( s.ovf_mem, nd, s.ovf_capacity, s.om );
    else carve( s.ovf_mem, nd, s.ovf_capacity, s.od );
    if( npart > 0 ) {
        if( nd == 3 ) {
            if( S->mixed ) k_stage<3, true><<<grid_for( npart, 256 ), 256, 0, st>>>( S->g, npart, pos, mom, weight, s.om, s.ovf_tile, s.count[1] );
            else k_stage<3, false><<<grid_for( npart, 256 ), 256, 0, st>>>( S->g, npart, pos, mom, weight, s.od, s.ovf_tile, s.count[1] );
        } else {
            if( S->mixed ) k_stage<2, true><<<grid_for( npart, 256 ), 256, 0, st>>>( S->g, npart, pos, mom, weight, s.om, s.ovf_tile, s.count[1] );
            else k_stage<2, false><<<grid_for( npart, 256 ), 256, 0, st>>>( S->g, npart, pos, mom, weight, s.od, s.ovf_tile, s.count[1] );
        }
        SG_LAUNCH_CHECK( "k_stage" );
    }
    int64_t total = 0;
    int r = layout_from_counts( S, s.count[1], s.cap, s.seg_start, &total, &s.max_cap, s.h_cap );
    if( r ) return r;
    r = refresh_order( S, s );
    if( r ) return r;
    r = alloc_species_buffers( S, s, std::max<int64_t>( total, 1 ) );
    if( r ) return r;
    SG_CUDA_TRY( cudaMemsetAsync( S->fill, 0, nt * sizeof( int ), st ) );
    if( S->mixed ) r = place_staged<true>( S, s, npart, s.om, s.ovf_tile, 0 );
    else r = place_staged<false>( S, s, npart, s.od, s.ovf_tile, 0 );
    if( r ) return r;
    SG_CUDA_TRY( cudaMemcpyAsync( s.count[0], S->fill, nt * sizeof( int ), cudaMemcpyDeviceToDevice, st ) );
    SG_CUDA_TRY( cudaStreamSynchronize( st ) );
    // the spill list only needs a fraction of the species once placed
    const int64_t spill_cap = std::max<int64_t>( 4096, npart / 16 );
    if( spill_cap < s.ovf_capacity ) {
        release( s.ovf_mem );
        release( s.ovf_tile );
        s.ovf_mem = nullptr;
        s.ovf_tile = nullptr;
        s.ovf_capacity = spill_cap;
        const size_t sbytes = S->mixed ? pbuf_bytes<true>( nd, spill_cap ) : pbuf_bytes<false>( nd, spill_cap );
        SG_CUDA_TRY( cudaMalloc( &s.ovf_mem, sbytes ) );
        SG_CUDA_TRY( cudaMalloc( &s.ovf_tile, spill_cap * sizeof( int ) ) );
        if( S->mixed ) carve( s.ovf_mem, nd, spill_cap, s.om );
        else carve( s.ovf_mem, nd, spill_cap, s.od );
    }
    s.cur = S->sp.size() > 1 ? S->sp[0].cur : 0;
    if( s.cur != 0 ) {
        // keep every species on the same buffer parity: move the data to buffer 1
        const size_t bytes = S->mixed ? pbuf_bytes<true>( nd, s.capacity ) : pbuf_bytes<false>( nd, s.capacity );
        SG_CUDA_TRY( cudaMemcpyAsync( s.mem[1], s.mem[0], bytes, cudaMemcpyDeviceToDevice, st ) );
        SG_CUDA_TRY( cudaMemcpyAsync( s.count[1], s.count[0], nt * sizeof( int ), cudaMemcpyDeviceToDevice, st ) );
        SG_CUDA_TRY( cudaStreamSynchronize( st ) );
    }
    drop_graphs( S );
    if( index ) *index = ( int )S->sp.size() - 1;
    return SG_OK;
}

int sg_sim_add_species( sg_sim *S, double mass, double charge, int pusher, int64_t npart, const double *pos,
                        const double *mom, const double *weight, int *index )
{
    SG_REQUIRE( S, "NULL simulation" );
    SG_REQUIRE( npart >= 0, "npart < 0" );
    const int nd = S->g.ndim;
    double *d = nullptr;
    const size_t bytes = ( size_t )( nd + 4 ) * ( size_t )std::max<int64_t>( npart, 1 ) * 8;
    SG_CUDA_TRY( cudaMalloc( &d, bytes ) );
    if( npart > 0 ) {
        SG_CUDA_TRY( cudaMemcpy( d, pos, nd * npart * 8, cudaMemcpyHostToDevice ) );
        SG_CUDA_TRY( cudaMemcpy( d + nd * npart, mom, 3 * npart * 8, cudaMemcpyHostToDevice ) );
        SG_CUDA_TRY( cudaMemcpy( d + ( nd + 3 ) * npart, weight, npart * 8, cudaMemcpyHostToDevice ) );
    }
    int r = sg_sim_add_species_device( S, mass, charge, pusher, npart, d, d + nd * npart, d + ( nd + 3 ) * npart, index );
    release( d );
    return r;
}

int sg_sim_field_shape( sg_sim *S, int comp, int *shape3 )
{
    SG_REQUIRE( S && shape3, "NULL argument" );
    SG_REQUIRE( comp >= 0 && comp < 12, "component out of range" );
    for( int d = 0; d < 3; d++ ) shape3[d] = S->fshape[comp][d];
    return SG_OK;
}

int sg_sim_set_field( sg_sim *S, int comp, const double *host )
{
    if( S ) S->energy_valid = false;
    SG_REQUIRE( S && host, "NULL argument" );
    SG_REQUIRE( comp >= 0 && comp < 12, "component out of range" );
    const int64_t n = S->fsize[comp];
    SG_CUDA_TRY( cudaStreamSynchronize( S->stream ) );
    S->pad_dirty = true;
    if( !S->mixed || felem( S, comp ) == 8 ) {
        SG_CUDA_TRY( cudaMemcpy( S->fptr[comp], host, n * 8, cudaMemcpyHostToDevice ) );
    } else {
        double *d = nullptr;
        SG_CUDA_TRY( cudaMalloc( &d, n * 8 ) );
        SG_CUDA_TRY( cudaMemcpy( d, host, n * 8, cudaMemcpyHostToDevice ) );
        k_convert<double, float><<<grid_for( n, 256 ), 256, 0, S->stream>>>( n, d, static_cast<float *>( S->fptr[comp] ) );
        SG_LAUNCH_CHECK( "k_convert" );
        if( comp < 3 && S->ecomp[comp] ) SG_CUDA_TRY( cudaMemsetAsync( S->ecomp[comp], 0, n * S->esz, S->stream ) );
        SG_CUDA_TRY( cudaStreamSynchronize( S->stream ) );
        release( d );
    }
    return SG_OK;
}

int sg_sim_get_field( sg_sim *S, int comp, double *host )
{
    SG_REQUIRE( S && host, "NULL argument" );
    SG_REQUIRE( comp >= 0 && comp < 12, "component out of range" );
    const int64_t n = S->fsize[comp];
    SG_CUDA_TRY( cudaStreamSynchronize( S->stream ) );
    if( !S->mixed || felem( S, comp ) == 8 ) {
        SG_CUDA_TRY( cudaMemcpy( host, S->fptr[comp], n * 8, cudaMemcpyDeviceToHost ) );
    } else {
        double *d = nullptr;
        SG_CUDA_TRY( cudaMalloc( &d, n * 8 ) );
        k_convert<float, double><<<grid_for( n, 256 ), 256, 0, S->stream>>>( n, static_cast<float *>( S->fptr[comp] ), d );
        SG_LAUNCH_CHECK( "k_convert" );
        SG_CUDA_TRY( cudaStreamSynchronize( S->stream ) );
        SG_CUDA_TRY( cudaMemcpy( host, d, n * 8, cudaMemcpyDeviceToHost ) );
        release( d );
    }
    return SG_OK;
}

// After the step enqueued on S->stream: waits for it, swaps the buffers, reads the
// status and removal counts, re-lays out spilled species and shifts the window.
// A finished step's flags (status, spills, removals; layout at d_flags): the error it
// raised, or the particles it removed and the re-layout of a species that spilled.
// removed: the removals to account (a batch passes its sums over its steps).
static int apply_step_flags( sg_sim *S, const int *flags, const int *removed )
{
    const int status = flags[0];
    if( status ) {
        return set_error( status, status == SG_ERR_BOUNDS ? "a particle moved more than one cell in a step or left its tile"
                                  : status == SG_ERR_ARG ? "a tile of the packed state exceeds its segment in the current layout"
                                                         : "the spill list overflowed (capacity too small)" );
    }
    for( size_t k = 0; k < S->sp.size(); k++ ) S->sp[k].npart -= removed[k];
    for( size_t k = 0; k < S->sp.size(); k++ ) {
        const int nspill = flags[1 + k];
        if( nspill > 0 ) {
            S->relayouts++;
            S->spilled += nspill;
            int r = relayout( S, S->sp[k], nspill );
            if( r ) return r;
        }
    }
    return SG_OK;
}

static int finish_step( sg_sim *S, bool moving )
{
    SG_CUDA_TRY( cudaStreamSynchronize( S->stream ) );
    for( auto &s : S->sp ) s.cur = 1 - s.cur;
    // stage times from the events recorded inside the step (external event nodes in a graph)
    if( cudaEventElapsedTime( &S->last_ms[0], S->ev[0], S->ev[1] ) != cudaSuccess ||
        cudaEventElapsedTime( &S->last_ms[1], S->ev[1], S->ev[2] ) != cudaSuccess ||
        cudaEventElapsedTime( &S->last_ms[2], S->ev[3], S->ev[2] ) != cudaSuccess ) {
        cudaGetLastError(); // timing is informative only; do not leave the error pending
        S->last_ms[0] = S->last_ms[1] = S->last_ms[2] = -1.0f;
    }
    int r = apply_step_flags( S, S->h_flags, S->h_flags + 1 + S->max_species );
    if( r ) return r;
    if( moving ) {
        int r = window_shift( S );
        if( r ) return r;
        S->win_x_moved += S->g.dx[0] * S->win_shift;
    }
    S->hstep++;
    return SG_OK;
}

// Whether the window moves at the end of step `step` (SimWindow::isMoving,
// SimWindow.cpp:93-96), with the window where it is now.
static bool window_moves_at( const sg_sim *S, int64_t step )
{
    const double time_dual = ( ( double )step + 1.5 ) * S->g.dt;
    return S->win_on && ( time_dual - S->win_t_start ) * S->win_velocity > S->win_x_moved;
}

// Up to `limit` steps (2 <= limit <= BATCH_STEPS, none of them moving the window) as one
// batched graph and one wait.  *done: the steps made (0 when batches are unavailable).
static int run_batch( sg_sim *S, int limit, int *done )
{
    *done = 0;
    const int parity = S->sp.empty() ? 0 : S->sp[0].cur;
    // the graph for the present parity, built when first needed (a batch of an even
    // number of steps ends on the parity it started from, so the other one is built
    // only after a batch a spill cut short)
    if( S->batch_parity < 0 ) S->batch_parity = parity;
    const int idx = parity == S->batch_parity ? 0 : 1;
    if( !S->batch[idx] ) {
        int r = build_batch( S, &S->batch[idx] );
        if( r ) return r;
        if( !S->batch[idx] ) {
            S->batch_unsupported = true;
            drop_graphs( S );
            return SG_OK;
        }
    }
    const int rec = batch_record_ints( S->max_species );
    S->h_batch[rec] = limit;
    SG_CUDA_TRY( cudaMemcpyAsync( S->d_batch + 2, S->h_batch + rec, sizeof( int ), cudaMemcpyHostToDevice, S->stream ) );
    SG_CUDA_TRY( cudaGraphLaunch( S->batch[idx], S->stream ) );
    SG_CUDA_TRY( cudaStreamSynchronize( S->stream ) );
    const int n = S->h_batch[1];
    if( n < 1 || n > limit ) return set_error( SG_ERR_CUDA, "batched step record out of range (%d of %d)", n, limit );
    for( auto &s : S->sp )
        if( n & 1 ) s.cur = 1 - s.cur;
    S->last_ms[0] = S->last_ms[1] = S->last_ms[2] = -1.0f; // no stage events inside a batch
    // the flags are those of the batch's last step, the removals its sums over the steps
    S->hstep += n - 1;
    int r = apply_step_flags( S, S->h_batch + 3 + S->max_species, S->h_batch + 3 );
    if( r ) return r;
    S->hstep++;
    S->batches++;
    S->batched_steps += n;
    *done = n;
    return SG_OK;
}

int sg_sim_step( sg_sim *S, int nsteps )
{
    if( S ) S->energy_valid = false;
    SG_REQUIRE( S, "NULL simulation" );
    SG_REQUIRE( nsteps >= 0, "nsteps < 0" );
    for( int it = 0; it < nsteps; ) {
        int rp = pad_fields( S, S->stream );
        if( rp ) return rp;
        // steps before the window's next move go in batches, with one wait per batch
        int limit = 0;
        if( S->cfg.use_graph && !S->batch_unsupported && nsteps - it > 1 && !S->sp.empty() ) {
            const int most = std::min( nsteps - it, BATCH_STEPS );
            while( limit < most && !window_moves_at( S, S->hstep + limit ) ) limit++;
        }
        if( limit > 1 ) {
            int done = 0;
            int r = run_batch( S, limit, &done );
            if( r ) return r;
            if( done > 0 ) {
                it += done;
                continue;
            }
        }
        it++;
        const int parity = S->sp.empty() ? 0 : S->sp[0].cur;
        // the window moves at the end of this step (SimWindow::isMoving, SimWindow.cpp:93-96);
        // the x boundaries of this step are then skipped (ElectroMagn.cpp:374)
        const bool moving = window_moves_at( S, S->hstep );
        if( moving ) {
            S->obc.side_mask = 0xC;
            int r = enqueue_step( S, S->stream );
            S->obc.side_mask = 0xF;
            if( r ) return r;
        } else if( S->cfg.use_graph ) {
            if( S->graph_parity < 0 ) {
                // capture both parities: the step from the current state and the one after it
                int r = capture( S, &S->graph[0] );
                if( r ) return r;
                for( auto &s : S->sp ) s.cur = 1 - s.cur;
                r = capture( S, &S->graph[1] );
                for( auto &s : S->sp ) s.cur = 1 - s.cur;
                if( r ) return r;
                S->graph_parity = parity;
            }
            SG_CUDA_TRY( cudaGraphLaunch( S->graph[parity == S->graph_parity ? 0 : 1], S->stream ) );
        } else {
            int r = enqueue_step( S, S->stream );
            if( r ) return r;
        }
        int r = finish_step( S, moving );
        if( r ) return r;
    }
    return SG_OK;
}

int sg_sim_set_moving_window( sg_sim *S, double time_start, double velocity_x, int shift_cells )
{
    SG_REQUIRE( S, "NULL simulation" );
    SG_REQUIRE( S->g.ndim == 2 && S->g.open[0], "the moving window needs a 2D grid with an open x axis" );
    SG_REQUIRE( shift_cells > 0 && shift_cells < S->g.N[0], "shift_cells must be in [1, %d)", S->g.N[0] );
    SG_REQUIRE( velocity_x >= 0.0, "velocity_x must not be negative" );
    if( !S->win_scratch ) {
        int64_t mx = 0;
        for( int c = 0; c < 12; c++ ) mx = std::max( mx, S->fsize[c] );
        SG_CUDA_TRY( cudaMalloc( &S->win_scratch, ( size_t )mx * 8 ) );
    }
    S->win_on = true;
    S->win_t_start = time_start;
    S->win_velocity = velocity_x;
    S->win_shift = shift_cells;
    return SG_OK;
}

int sg_sim_window_state( sg_sim *S, int64_t *n_moved, double *x_moved, int64_t *shifts )
{
    SG_REQUIRE( S, "NULL simulation" );
    if( n_moved ) *n_moved = S->win_n_moved;
    if( x_moved ) *x_moved = S->win_x_moved;
    if( shifts ) *shifts = S->win_shifts;
    return SG_OK;
}

int sg_sim_set_species_profile( sg_sim *S, int species, const double *profile, int ppc, double temperature,
                                uint64_t seed )
{
    SG_REQUIRE( S && profile, "NULL argument" );
    SG_REQUIRE( species >= 0 && species < ( int )S->sp.size(), "species %d out of range", species );
    const int nd = S->g.ndim;
    int c = 1;
    while( ( nd == 2 ? c * c : c * c * c ) < ppc ) c++;
    SG_REQUIRE( ppc > 0 && ( nd == 2 ? c * c : c * c * c ) == ppc,
                "regular positions need ppc = c^%d particles per cell (got %d)", nd, ppc );
    SG_REQUIRE( temperature >= 0.0, "temperature must not be negative" );
    SG_REQUIRE( profile[2] >= 0.0 && profile[4] >= 0.0, "slopes must not be negative" );
    SpeciesState &s = S->sp[species];
    InjectParams &ip = s.inj;
    for( int k = 0; k < 5; k++ ) ip.prof[k] = profile[k];
    double vol = 1.0;
    for( int d = 0; d < nd; d++ ) vol *= S->g.dx[d];
    ip.vol = vol;
    ip.ppc = ppc;
    ip.c = c;
    ip.invc = 1.0 / ( double )c;
    ip.sqrt_temp = std::sqrt( temperature );
    ip.seed = ( unsigned long long )seed;
    s.inject = true;
    return SG_OK;
}

int sg_sim_set_species_radiation( sg_sim *S, int species, const sg_rad_tables *tables, const sg_mlp *mlp,
                                  uint32_t seed )
{
    SG_REQUIRE( S && tables, "NULL argument" );
    SG_REQUIRE( species >= 0 && species < ( int )S->sp.size(), "species %d out of range", species );
    SG_REQUIRE( S->mixed && S->g.ndim == 2, "radiation in the resident step needs the 2D mixed form" );
    SpeciesState &s = S->sp[species];
    SG_CUDA_TRY( cudaStreamSynchronize( S->stream ) );
    if( !s.radiates ) {
        s.radiates = true;
        int r = alloc_tau( S, s, s.capacity );
        if( r ) return r;
        SG_CUDA_TRY( cudaMalloc( &s.ovf_tau, ( size_t )std::max<int64_t>( s.ovf_capacity, 1 ) * sizeof( float ) ) );
        s.om.tau = static_cast<float *>( s.ovf_tau );
        // optical depths start spent: the first step draws them (tau = -1, RadiationMonteCarlo.cpp:337)
        for( int b = 0; b < 2; b++ ) {
            k_fill<float><<<grid_for( std::max<int64_t>( s.capacity, 1 ), 256 ), 256, 0, S->stream>>>( s.capacity, s.bm[b].tau, -1.0f );
            SG_LAUNCH_CHECK( "k_fill" );
        }
        SG_CUDA_TRY( cudaMalloc( &s.d_rad, 2 * sizeof( double ) ) );
        SG_CUDA_TRY( cudaMemsetAsync( s.d_rad, 0, 2 * sizeof( double ), S->stream ) );
        if( !S->d_rad_step ) {
            SG_CUDA_TRY( cudaMalloc( &S->d_rad_step, sizeof( int64_t ) ) );
            SG_CUDA_TRY( cudaMemsetAsync( S->d_rad_step, 0, sizeof( int64_t ), S->stream ) );
        }
        SG_CUDA_TRY( cudaStreamSynchronize( S->stream ) );
    }
    s.rad_tables = tables;
    s.rad_mlp = mlp;
    s.rad_seed = seed;
    drop_graphs( S );
    return SG_OK;
}

int sg_sim_radiation_stats( sg_sim *S, int species, double *radiated, unsigned long long *emissions )
{
    SG_REQUIRE( S, "NULL simulation" );
    SG_REQUIRE( species >= 0 && species < ( int )S->sp.size(), "species %d out of range", species );
    const SpeciesState &s = S->sp[species];
    SG_REQUIRE( s.radiates, "species %d does not radiate", species );
    double h[2] = { 0.0, 0.0 };
    SG_CUDA_TRY( cudaMemcpyAsync( h, s.d_rad, sizeof( h ), cudaMemcpyDeviceToHost, S->stream ) );
    SG_CUDA_TRY( cudaStreamSynchronize( S->stream ) );
    if( radiated ) *radiated = h[0];
    if( emissions ) std::memcpy( emissions, &h[1], sizeof( unsigned long long ) );
    return SG_OK;
}

int sg_sim_set_species_photons( sg_sim *S, int species, int sampling, double gamma_threshold, int max_emissions,
                                int64_t capacity )
{
    SG_REQUIRE( S, "NULL simulation" );
    SG_REQUIRE( species >= 0 && species < ( int )S->sp.size(), "species %d out of range", species );
    SpeciesState &s = S->sp[species];
    SG_REQUIRE( s.radiates, "species %d does not radiate (sg_sim_set_species_radiation first)", species );
    SG_REQUIRE( capacity >= 0, "capacity < 0" );
    SG_REQUIRE( capacity == 0 || ( sampling >= 1 && max_emissions >= 1 ), "sampling and max_emissions must be >= 1" );
    SG_CUDA_TRY( cudaStreamSynchronize( S->stream ) );
    drop_graphs( S ); // the pass and the step hold the store's pointers
    release( s.ph_mem );
    release( s.ph_count );
    s.ph_mem = nullptr;
    s.ph_count = nullptr;
    s.ph_cap = 0;
    if( capacity == 0 ) return SG_OK;
    if( cudaMalloc( &s.ph_mem, ( size_t )capacity * 8 * sizeof( double ) ) != cudaSuccess ||
        cudaMalloc( &s.ph_count, sizeof( unsigned long long ) ) != cudaSuccess ) {
        release( s.ph_mem );
        s.ph_mem = nullptr;
        return set_error( SG_ERR_NOMEM, "cannot allocate a store of %lld photons", ( long long )capacity );
    }
    SG_CUDA_TRY( cudaMemsetAsync( s.ph_count, 0, sizeof( unsigned long long ), S->stream ) );
    s.ph_cap = capacity;
    s.ph_sampling = sampling;
    s.ph_threshold = gamma_threshold;
    s.ph_max_emissions = max_emissions;
    SG_CUDA_TRY( cudaStreamSynchronize( S->stream ) );
    return SG_OK;
}

int sg_sim_get_photons( sg_sim *S, int species, int64_t *count, double *pos, double *mom, double *weight, double *chi,
                        double *tau )
{
    SG_REQUIRE( S, "NULL simulation" );
    SG_REQUIRE( species >= 0 && species < ( int )S->sp.size(), "species %d out of range", species );
    const SpeciesState &s = S->sp[species];
    SG_REQUIRE( s.ph_mem, "species %d has no photon store (sg_sim_set_species_photons)", species );
    unsigned long long c = 0;
    SG_CUDA_TRY( cudaMemcpyAsync( &c, s.ph_count, sizeof( c ), cudaMemcpyDeviceToHost, S->stream ) );
    SG_CUDA_TRY( cudaStreamSynchronize( S->stream ) );
    if( count ) *count = ( int64_t )c;
    const int64_t n = std::min<int64_t>( ( int64_t )c, s.ph_cap );
    const size_t b = ( size_t )n * sizeof( double );
    const int64_t cap = s.ph_cap;
    for( int d = 0; pos && d < 2; d++ ) SG_CUDA_TRY( cudaMemcpy( pos + d * n, s.ph_mem + d * cap, b, cudaMemcpyDeviceToHost ) );
    for( int d = 0; mom && d < 3; d++ )
        SG_CUDA_TRY( cudaMemcpy( mom + d * n, s.ph_mem + ( 2 + d ) * cap, b, cudaMemcpyDeviceToHost ) );
    if( weight ) SG_CUDA_TRY( cudaMemcpy( weight, s.ph_mem + 5 * cap, b, cudaMemcpyDeviceToHost ) );
    if( chi ) SG_CUDA_TRY( cudaMemcpy( chi, s.ph_mem + 6 * cap, b, cudaMemcpyDeviceToHost ) );
    if( tau ) SG_CUDA_TRY( cudaMemcpy( tau, s.ph_mem + 7 * cap, b, cudaMemcpyDeviceToHost ) );
    return SG_OK;
}

int sg_sim_fill_species( sg_sim *S, int species, int x0_cell, int x1_cell )
{
    if( S ) S->energy_valid = false;
    SG_REQUIRE( S, "NULL simulation" );
    SG_REQUIRE( species >= 0 && species < ( int )S->sp.size(), "species %d out of range", species );
    SpeciesState &s = S->sp[species];
    SG_REQUIRE( s.inject, "species %d has no profile (sg_sim_set_species_profile)", species );
    SG_REQUIRE( 0 <= x0_cell && x0_cell <= x1_cell && x1_cell <= S->g.N[0], "cells [%d, %d) out of [0, %d]", x0_cell,
                x1_cell, S->g.N[0] );
    SG_CUDA_TRY( cudaStreamSynchronize( S->stream ) );
    return rebuild_species( S, s, 0, x0_cell, x1_cell );
}

int sg_sim_add_laser_gaussian2d( sg_sim *S, const double *p )
{
    SG_REQUIRE( S && p, "NULL argument" );
    SG_REQUIRE( S->g.ndim == 2 && S->g.open[0], "a Gaussian 2D laser needs a 2D grid with an open x axis" );
    SG_REQUIRE( S->obc.nlaser < MAX_LASERS, "at most %d lasers", MAX_LASERS );
    const double a0 = p[0], omega = p[1], waist = p[2], fx = p[3], fy = p[4], pphi = p[5], ell = p[6];
    SG_REQUIRE( omega > 0.0 && waist > 0.0 && p[11] > 0.0, "omega, waist and fwhm must be positive" );
    // LaserGaussian2D (pyprofiles.py:507-569) with transformPolarization (:458-468): its
    // [dephasing, A1, A2] is unpacked as (dephasing, amplitudeZ, amplitudeY), so the By
    // profile takes A2 and the Bz profile A1
    const double e2 = ell * ell;
    const double pp = ( 1.0 - e2 ) * std::sin( 2.0 * pphi ) / 2.0;
    const double dephasing = std::atan2( ell, pp );
    const double amplitude = std::sqrt( 1.0 / ( 1.0 + e2 ) );
    const double c2 = std::cos( pphi ) * std::cos( pphi ), s2 = 1.0 - c2;
    LaserG2 L{};
    L.omega = omega;
    L.fy = fy;
    L.amp[0] = amplitude * std::sqrt( s2 + e2 * c2 ) * a0 * omega;
    L.amp[1] = amplitude * std::sqrt( c2 + e2 * s2 ) * a0 * omega;
    L.delay[0] = 0.0;
    L.delay[1] = dephasing;
    L.phase_offset = p[7];
    const double Zr = omega * waist * waist / 2.0;
    const double w = std::sqrt( 1.0 / ( 1.0 + ( fx / Zr ) * ( fx / Zr ) ) );
    L.invWaist2 = ( w / waist ) * ( w / waist );
    L.coeff = -omega * fx * w * w / ( 2.0 * Zr * Zr );
    L.sqrtw = std::sqrt( w );
    L.t_start = p[8];
    L.t_end = p[8] + p[9];
    L.t_center = p[10];
    L.t_order = p[12];
    L.t_invsigma = 1.0 / ( std::pow( 0.5 * p[11], p[12] ) / std::log( 2.0 ) );
    S->obc.laser[S->obc.nlaser++] = L;
    drop_graphs( S ); // the boundary kernel takes the lasers by value
    return SG_OK;
}

int sg_sim_layout_stats( sg_sim *S, int64_t *relayouts, int64_t *spilled )
{
    SG_REQUIRE( S, "NULL simulation" );
    if( relayouts ) *relayouts = S->relayouts;
    if( spilled ) *spilled = S->spilled;
    return SG_OK;
}

int sg_sim_batch_stats( sg_sim *S, int64_t *batches, int64_t *steps, int *unsupported )
{
    SG_REQUIRE( S, "NULL simulation" );
    if( batches ) *batches = S->batches;
    if( steps ) *steps = S->batched_steps;
    if( unsupported ) *unsupported = S->batch_unsupported ? 1 : 0;
    return SG_OK;
}

int sg_sim_last_timing( sg_sim *S, double *ms_particles, double *ms_fields, double *ms_total, int *launches_per_step )
{
    SG_REQUIRE( S, "NULL simulation" );
    if( ms_particles ) *ms_particles = S->last_ms[0];
    if( ms_fields ) *ms_fields = S->last_ms[1];
    if( ms_total ) *ms_total = S->last_ms[2];
    if( launches_per_step ) *launches_per_step = S->launches_per_step;
    return SG_OK;
}

int sg_sim_species_count( sg_sim *S, int species, int64_t *npart )
{
    SG_REQUIRE( S && npart, "NULL argument" );
    SG_REQUIRE( species >= 0 && species < ( int )S->sp.size(), "no species %d", species );
    SpeciesState &s = S->sp[species];
    const int nt = S->g.ntiles;
    std::vector<int> c( nt );
    SG_CUDA_TRY( cudaStreamSynchronize( S->stream ) );
    SG_CUDA_TRY( cudaMemcpy( c.data(), s.count[s.cur], nt * sizeof( int ), cudaMemcpyDeviceToHost ) );
    int64_t n = 0;
    for( int v : c ) n += v;
    *npart = n;
    return SG_OK;
}

int sg_sim_get_species( sg_sim *S, int species, double *pos, double *mom, double *weight )
{
    SG_REQUIRE( S && pos && mom && weight, "NULL argument" );
    SG_REQUIRE( species >= 0 && species < ( int )S->sp.size(), "no species %d", species );
    SpeciesState &s = S->sp[species];
    const int nt = S->g.ntiles, nd = S->g.ndim;
    int64_t n = 0;
    int r = sg_sim_species_count( S, species, &n );
    if( r ) return r;
    int64_t *off = nullptr;
    double *d = nullptr;
    SG_CUDA_TRY( cudaMalloc( &off, nt * sizeof( int64_t ) ) );
    SG_CUDA_TRY( cudaMalloc( &d, ( size_t )( nd + 4 ) * std::max<int64_t>( n, 1 ) * 8 ) );
    r = exclusive_scan<int>( s.count[s.cur], nt, off, S->scan_scratch, S->stream );
    if( r ) return r;
    if( nd == 3 ) {
        if( S->mixed ) k_export<3, true><<<nt, 128, 0, S->stream>>>( S->g, nt, s.seg_start, s.count[s.cur], off, s.bm[s.cur], n, d, d + nd * n, d + ( nd + 3 ) * n );
        else k_export<3, false><<<nt, 128, 0, S->stream>>>( S->g, nt, s.seg_start, s.count[s.cur], off, s.bd[s.cur], n, d, d + nd * n, d + ( nd + 3 ) * n );
    } else {
        if( S->mixed ) k_export<2, true><<<nt, 128, 0, S->stream>>>( S->g, nt, s.seg_start, s.count[s.cur], off, s.bm[s.cur], n, d, d + nd * n, d + ( nd + 3 ) * n );
        else k_export<2, false><<<nt, 128, 0, S->stream>>>( S->g, nt, s.seg_start, s.count[s.cur], off, s.bd[s.cur], n, d, d + nd * n, d + ( nd + 3 ) * n );
    }
    SG_LAUNCH_CHECK( "k_export" );
    SG_CUDA_TRY( cudaStreamSynchronize( S->stream ) );
    SG_CUDA_TRY( cudaMemcpy( pos, d, nd * n * 8, cudaMemcpyDeviceToHost ) );
    SG_CUDA_TRY( cudaMemcpy( mom, d + nd * n, 3 * n * 8, cudaMemcpyDeviceToHost ) );
    SG_CUDA_TRY( cudaMemcpy( weight, d + ( nd + 3 ) * n, n * 8, cudaMemcpyDeviceToHost ) );
    release( off );
    release( d );
    return SG_OK;
}

int sg_sim_state_bytes( sg_sim *S, int species, size_t *bytes )
{
    SG_REQUIRE( S && bytes, "NULL argument" );
    SG_REQUIRE( species >= 0 && species < ( int )S->sp.size(), "no species %d", species );
    const SpeciesState &s = S->sp[species];
    *bytes = S->mixed ? pbuf_bytes<true>( S->g.ndim, s.capacity ) : pbuf_bytes<false>( S->g.ndim, s.capacity );
    return SG_OK;
}

int sg_sim_copy_state( sg_sim *S, int species, void *host, int to_device )
{
    if( S ) S->energy_valid = false;
    SG_REQUIRE( S && host, "NULL argument" );
    SG_REQUIRE( species >= 0 && species < ( int )S->sp.size(), "no species %d", species );
    SpeciesState &s = S->sp[species];
    size_t bytes = 0;
    sg_sim_state_bytes( S, species, &bytes );
    if( to_device ) SG_CUDA_TRY( cudaMemcpyAsync( s.mem[s.cur], host, bytes, cudaMemcpyHostToDevice, S->stream ) );
    else SG_CUDA_TRY( cudaMemcpyAsync( host, s.mem[s.cur], bytes, cudaMemcpyDeviceToHost, S->stream ) );
    return SG_OK;
}

int sg_sim_packed_bytes( sg_sim *S, int species, size_t *bytes )
{
    SG_REQUIRE( S && bytes, "NULL argument" );
    SG_REQUIRE( species >= 0 && species < ( int )S->sp.size(), "no species %d", species );
    const int nd = S->g.ndim;
    const size_t per = S->mixed ? ( size_t )( 4 + 4 * nd + 16 ) : ( size_t )( 8 * nd + 32 );
    *bytes = packed_header_bytes( S->g.ntiles ) + per * ( size_t )S->sp[species].npart;
    return SG_OK;
}

// staging buffer of at least `bytes` on the device
static int packed_staging( sg_sim *S, size_t bytes )
{
    if( S->pack_bytes >= bytes ) return SG_OK;
    release( S->pack_mem );
    S->pack_mem = nullptr;
    S->pack_bytes = 0;
    SG_CUDA_TRY( cudaMalloc( &S->pack_mem, bytes ) );
    S->pack_bytes = bytes;
    return SG_OK;
}

int sg_sim_pack_state( sg_sim *S, int species, void *host )
{
    SG_REQUIRE( S && host, "NULL argument" );
    SG_REQUIRE( species >= 0 && species < ( int )S->sp.size(), "no species %d", species );
    SpeciesState &s = S->sp[species];
    const int nt = S->g.ntiles, nd = S->g.ndim;
    size_t bytes = 0;
    int r = sg_sim_packed_bytes( S, species, &bytes );
    if( r ) return r;
    r = packed_staging( S, bytes );
    if( r ) return r;
    char *stg = static_cast<char *>( S->pack_mem );
    const int64_t n = s.npart;
    r = exclusive_scan<int>( s.count[s.cur], nt, S->tmp_start, S->scan_scratch, S->stream );
    if( r ) return r;
    SG_CUDA_TRY( cudaMemcpyAsync( stg, &s.npart, 8, cudaMemcpyHostToDevice, S->stream ) );
    if( S->mixed ) k_pack<true, true><<<nt, 128, 0, S->stream>>>( nd, nt, s.seg_start, s.cap, s.count[s.cur], S->tmp_start, s.bm[s.cur], n, stg, S->d_flags, 0 );
    else k_pack<false, true><<<nt, 128, 0, S->stream>>>( nd, nt, s.seg_start, s.cap, s.count[s.cur], S->tmp_start, s.bd[s.cur], n, stg, S->d_flags, 0 );
    SG_LAUNCH_CHECK( "k_pack" );
    SG_CUDA_TRY( cudaMemcpyAsync( host, stg, bytes, cudaMemcpyDeviceToHost, S->stream ) );
    return SG_OK;
}

int sg_sim_unpack_state( sg_sim *S, int species, const void *host )
{
    if( S ) S->energy_valid = false;
    SG_REQUIRE( S && host, "NULL argument" );
    SG_REQUIRE( species >= 0 && species < ( int )S->sp.size(), "no species %d", species );
    SpeciesState &s = S->sp[species];
    const int nt = S->g.ntiles, nd = S->g.ndim;
    int64_t n = 0;
    std::memcpy( &n, host, 8 );
    SG_REQUIRE( n == s.npart, "the packed state holds %lld particles, the species %lld", ( long long )n,
                ( long long )s.npart );
    size_t bytes = 0;
    int r = sg_sim_packed_bytes( S, species, &bytes );
    if( r ) return r;
    r = packed_staging( S, bytes );
    if( r ) return r;
    char *stg = static_cast<char *>( S->pack_mem );
    SG_CUDA_TRY( cudaMemcpyAsync( stg, host, bytes, cudaMemcpyHostToDevice, S->stream ) );
    r = exclusive_scan<int>( reinterpret_cast<const int *>( stg + 8 ), nt, S->tmp_start, S->scan_scratch, S->stream );
    if( r ) return r;
    SG_CUDA_TRY( cudaMemsetAsync( S->d_flags, 0, sizeof( int ), S->stream ) );
    if( S->mixed ) k_pack<true, false><<<nt, 128, 0, S->stream>>>( nd, nt, s.seg_start, s.cap, s.count[s.cur], S->tmp_start, s.bm[s.cur], n, stg, S->d_flags, 0 );
    else k_pack<false, false><<<nt, 128, 0, S->stream>>>( nd, nt, s.seg_start, s.cap, s.count[s.cur], S->tmp_start, s.bd[s.cur], n, stg, S->d_flags, 0 );
    SG_LAUNCH_CHECK( "k_pack" );
    SG_CUDA_TRY( cudaMemcpyAsync( S->h_flags, S->d_flags, sizeof( int ), cudaMemcpyDeviceToHost, S->stream ) );
    SG_CUDA_TRY( cudaStreamSynchronize( S->stream ) );
    if( S->h_flags[0] ) return set_error( SG_ERR_ARG, "a tile of the packed state exceeds its segment in the current layout" );
    return SG_OK;
}

// Tile ranges of a streamed step, in processing order, from the packed particle offsets
// hoff[0..nt] (tile order).  Returns whether the ranges can be packed while stepping:
// that needs the particle count to stay (no open boundary removes any) and three x-slabs
// of tiles at least.  The last x-slab is then range 0 and steps first: the first slab
// receives from it across the periodic boundary, and would otherwise be final only at the
// end, with every packed offset behind it.  The other `chunks` ranges cut the remaining
// tiles at about equal particle counts.  A tile receives from its own x-slab and the two
// beside it (the y and z wraps stay inside a slab), so range j is final once every tile
// up to the end of the slab after its last tile has stepped: pack_after[j] is the first
// range that reaches there.
static bool plan_stream( int nd, const int *ntiles, bool periodic, const std::vector<int64_t> &hoff, int chunks,
                         std::vector<int> &ta, std::vector<int> &tb, std::vector<int> &pack_after )
{
    const int nt = ( int )hoff.size() - 1;
    const int slab = nd == 3 ? ntiles[1] * ntiles[2] : ntiles[1];
    const bool pack = periodic && ntiles[0] >= 3;
    const int body = pack ? nt - slab : nt;
    ta.clear();
    tb.clear();
    pack_after.clear();
    if( pack ) {
        ta.push_back( body );
        tb.push_back( nt );
    }
    for( int c = 0, t = 0; c < chunks; c++ ) {
        const int t0 = t;
        const int64_t target = hoff[body] / chunks * ( c + 1 );
        while( t < body && ( c == chunks - 1 || hoff[t] < target ) ) t++;
        ta.push_back( t0 );
        tb.push_back( t );
    }
    if( !pack ) return false;
    const int nr = ( int )ta.size();
    pack_after.assign( nr, nr - 1 );
    for( int j = 1; j < nr; j++ ) {
        const int need = std::min( body, ( std::max( tb[j] - 1, 0 ) / slab + 2 ) * slab );
        int q = j;
        while( q < nr - 1 && tb[q] < need ) q++;
        pack_after[j] = q;
    }
    pack_after[0] = nr - 1; // the last slab receives from the range before it
    return true;
}

int sg_stream_ranges( int ndim, const int *ntiles, int periodic, const int *counts, int chunks, int *ta, int *tb,
                      int *pack_after, int *nranges )
{
    SG_REQUIRE( ntiles && counts && ta && tb && pack_after && nranges, "NULL argument" );
    SG_REQUIRE( ndim == 2 || ndim == 3, "ndim must be 2 or 3" );
    SG_REQUIRE( chunks >= 1 && chunks <= 64, "chunks must be in [1, 64], got %d", chunks );
    int64_t nt = 1;
    for( int d = 0; d < ndim; d++ ) {
        SG_REQUIRE( ntiles[d] >= 1, "ntiles[%d] < 1", d );
        nt *= ntiles[d];
    }
    SG_REQUIRE( nt < ( int64_t )1 << 30, "too many tiles" );
    std::vector<int64_t> hoff( nt + 1, 0 );
    for( int64_t t = 0; t < nt; t++ ) {
        SG_REQUIRE( counts[t] >= 0, "tile %lld has a negative count", ( long long )t );
        hoff[t + 1] = hoff[t] + counts[t];
    }
    std::vector<int> a, b, p;
    const bool pack = plan_stream( ndim, ntiles, periodic != 0, hoff, chunks, a, b, p );
    for( size_t j = 0; j < a.size(); j++ ) {
        ta[j] = a[j];
        tb[j] = b[j];
        pack_after[j] = pack ? p[j] : -1;
    }
    *nranges = ( int )a.size();
    return SG_OK;
}

int enqueue_energy( sg_sim *S, cudaStream_t st, bool next );

// Particles [p0, p1) of every plane of a packed state (planes of n values of esz bytes
// after an hdr-byte header) between host and device: one strided copy where the planes'
// distance is within the device's pitch limit, else one copy per plane.
static cudaError_t copy_planes( char *dst, const char *src, size_t hdr, int planes, int64_t n, int64_t p0, int64_t p1,
                                size_t esz, size_t max_pitch, cudaMemcpyKind kind, cudaStream_t st )
{
    if( p1 <= p0 ) return cudaSuccess;
    const size_t pitch = ( size_t )n * esz, o = hdr + ( size_t )p0 * esz, w = ( size_t )( p1 - p0 ) * esz;
    if( pitch <= max_pitch ) return cudaMemcpy2DAsync( dst + o, pitch, src + o, pitch, w, ( size_t )planes, kind, st );
    for( int k = 0; k < planes; k++ ) {
        const cudaError_t e = cudaMemcpyAsync( dst + o + k * pitch, src + o + k * pitch, w, kind, st );
        if( e != cudaSuccess ) return e;
    }
    return cudaSuccess;
}

int sg_sim_step_host( sg_sim *S, int species, const void *host_in, void *host_out, int chunks )
{
    SG_REQUIRE( S && host_in && host_out, "NULL argument" );
    SG_REQUIRE( species >= 0 && species < ( int )S->sp.size(), "no species %d", species );
    SG_REQUIRE( chunks >= 1 && chunks <= 64, "chunks must be in [1, 64], got %d", chunks );
    SpeciesState &s = S->sp[species];
    SG_REQUIRE( !s.radiates, "a radiating species does not stream: its radiation pass reads every particle before the push" );
    S->energy_valid = false;
    const double time_dual = ( ( double )S->hstep + 1.5 ) * S->g.dt;
    const bool moving = S->win_on && ( time_dual - S->win_t_start ) * S->win_velocity > S->win_x_moved;
    SG_REQUIRE( !moving, "the window moves in this step (the state size changes): unpack, step and pack instead" );
    // a pack_state into host_in may still be in flight on the simulation's stream
    SG_CUDA_TRY( cudaStreamSynchronize( S->stream ) );
    const char *hin = static_cast<const char *>( host_in );
    int64_t n = 0;
    std::memcpy( &n, hin, 8 );
    SG_REQUIRE( n == s.npart, "the packed state holds %lld particles, the species %lld", ( long long )n,
                ( long long )s.npart );
    const int nt = S->g.ntiles, nd = S->g.ndim;
    const int *hc = reinterpret_cast<const int *>( hin + 8 );
    std::vector<int64_t> &hoff = S->h_off;
    hoff.resize( ( size_t )nt + 1 );
    hoff[0] = 0;
    for( int t = 0; t < nt; t++ ) {
        SG_REQUIRE( hc[t] >= 0, "tile %d of the packed state has a negative count", t );
        hoff[t + 1] = hoff[t] + hc[t];
    }
    SG_REQUIRE( hoff[nt] == n, "the packed tile counts sum to %lld, the header says %lld", ( long long )hoff[nt], ( long long )n );
    // The unpack would refuse a tile over its segment, but only after the copy out of
    // earlier ranges had begun, and host_out may be host_in: check before any copy.
    SG_REQUIRE( ( int )s.h_cap.size() == nt, "no host copy of the segment layout" );
    for( int t = 0; t < nt; t++ )
        if( hc[t] > s.h_cap[t] )
            return set_error( SG_ERR_ARG, "tile %d of the packed state holds %d particles, more than its segment (%d) in the current layout",
                              t, hc[t], s.h_cap[t] );

    StreamIn in;
    in.species = species;
    in.n = n;
    bool periodic = true;
    for( int d = 0; d < nd; d++ ) periodic = periodic && !S->g.open[d];
    in.pack = plan_stream( nd, S->g.nt, periodic, hoff, chunks, in.ta, in.tb, in.pack_after );
    const int nr = ( int )in.ta.size();

    size_t bytes = 0;
    int r = sg_sim_packed_bytes( S, species, &bytes );
    if( r ) return r;
    r = packed_staging( S, bytes );
    if( r ) return r;
    if( !S->copy_stream ) SG_CUDA_TRY( cudaStreamCreateWithFlags( &S->copy_stream, cudaStreamNonBlocking ) );
    if( !S->max_pitch ) {
        int dev = 0, mp = 0;
        SG_CUDA_TRY( cudaGetDevice( &dev ) );
        SG_CUDA_TRY( cudaDeviceGetAttribute( &mp, cudaDevAttrMaxPitch, dev ) );
        S->max_pitch = ( size_t )( mp > 0 ? mp : 1 );
    }
    while( ( int )S->copy_ev.size() < 2 * nr + 3 ) {
        cudaEvent_t e = nullptr;
        SG_CUDA_TRY( cudaEventCreate( &e ) ); // timed: the stage times of the step
        S->copy_ev.push_back( e );
    }
    if( in.pack ) {
        if( S->pack_out_cap < bytes ) {
            release( S->pack_out_mem );
            S->pack_out_mem = nullptr;
            S->pack_out_cap = 0;
            SG_CUDA_TRY( cudaMalloc( &S->pack_out_mem, bytes ) );
            S->pack_out_cap = bytes;
        }
        if( !S->pack_off ) SG_CUDA_TRY( cudaMalloc( &S->pack_off, ( size_t )nt * sizeof( int64_t ) ) );
        if( !S->h_chunk_end ) {
            SG_CUDA_TRY( cudaHostAlloc( &S->h_chunk_end, 2 * 65 * sizeof( int64_t ), cudaHostAllocMapped ) );
            SG_CUDA_TRY( cudaHostGetDevicePointer( reinterpret_cast<void **>( &S->d_chunk_end ), S->h_chunk_end, 0 ) );
        }
        if( !S->out_stream ) SG_CUDA_TRY( cudaStreamCreateWithFlags( &S->out_stream, cudaStreamNonBlocking ) );
        for( int j = 0; j < nr; j++ ) S->h_chunk_end[2 * j] = S->h_chunk_end[2 * j + 1] = n;
    }
    char *stg = static_cast<char *>( S->pack_mem );
    const size_t hdr = packed_header_bytes( nt ), esz = S->mixed ? 4 : 8;
    const int planes = S->mixed ? 1 + nd + 4 : nd + 4;
    cudaStream_t cs = S->copy_stream;
    // the staging buffer is free once the work already queued on the simulation's stream is done
    SG_CUDA_TRY( cudaEventRecord( S->copy_ev[0], S->stream ) );
    SG_CUDA_TRY( cudaStreamWaitEvent( cs, S->copy_ev[0], 0 ) );
    SG_CUDA_TRY( cudaMemcpyAsync( stg, hin, 8 + 4 * ( size_t )nt, cudaMemcpyHostToDevice, cs ) );
    SG_CUDA_TRY( cudaEventRecord( S->copy_ev[1], cs ) );
    for( int j = 0; j < nr; j++ ) {
        const int64_t p0 = hoff[in.ta[j]], p1 = hoff[in.tb[j]];
        SG_CUDA_TRY( copy_planes( stg, hin, hdr, planes, n, p0, p1, esz, S->max_pitch, cudaMemcpyHostToDevice, cs ) );
        SG_CUDA_TRY( cudaEventRecord( S->copy_ev[2 + j], cs ) );
    }
    r = pad_fields( S, S->stream );
    if( r == SG_OK ) r = enqueue_step( S, S->stream, &in );
    // the energy sums of the new state run while the last ranges are copied out
    if( r == SG_OK && in.pack ) r = enqueue_energy( S, S->stream, true );
    if( r ) {
        cudaStreamSynchronize( cs );
        cudaStreamSynchronize( S->stream );
        return r;
    }
    char *hout = static_cast<char *>( host_out );
    if( in.pack ) {
        // copy each range out as soon as it is packed: the link carries both directions at once
        std::vector<int> order( nr );
        for( int j = 0; j < nr; j++ ) order[j] = j;
        std::stable_sort( order.begin(), order.end(), [&]( int x, int y ) { return in.pack_after[x] < in.pack_after[y]; } );
        const char *ostg = static_cast<const char *>( S->pack_out_mem );
        int64_t copied = 0;
        bool valid = true;
        cudaError_t e = cudaSuccess;
        for( int j : order ) {
            e = cudaEventSynchronize( S->copy_ev[2 + nr + j] );
            if( e != cudaSuccess ) break;
            if( in.tb[j] <= in.ta[j] ) continue;
            const int64_t p0 = S->h_chunk_end[2 * j], p1 = S->h_chunk_end[2 * j + 1];
            if( p0 < 0 || p1 < p0 || p1 > n ) {
                valid = false; // not a packing of n particles: the full pack below redoes it
                continue;
            }
            copied += p1 - p0;
            // host_out may be host_in: first finish the copy in of every range whose input this overwrites
            int last_in = -1;
            for( int i = 0; i < nr; i++ )
                if( hoff[in.ta[i]] < p1 && hoff[in.tb[i]] > p0 ) last_in = std::max( last_in, i );
            if( last_in >= 0 ) e = cudaStreamWaitEvent( S->out_stream, S->copy_ev[2 + last_in], 0 );
            if( e == cudaSuccess )
                e = copy_planes( hout, ostg, hdr, planes, n, p0, p1, esz, S->max_pitch, cudaMemcpyDeviceToHost, S->out_stream );
            if( e != cudaSuccess ) break;
        }
        if( e == cudaSuccess ) e = cudaMemcpyAsync( hout + 8, ostg + 8, 4 * ( size_t )nt, cudaMemcpyDeviceToHost, S->out_stream );
        if( e == cudaSuccess ) e = cudaEventRecord( S->copy_ev[2 + 2 * nr], S->out_stream );
        if( e == cudaSuccess ) e = cudaStreamSynchronize( S->out_stream );
        if( e != cudaSuccess ) {
            cudaStreamSynchronize( S->stream );
            return cuda_fail( e, "streamed step copy-out", __FILE__, __LINE__ );
        }
        r = finish_step( S, false );
        if( r ) return r;
        const cudaEvent_t marks[4] = { S->copy_ev[1 + nr], S->ev[1], S->copy_ev[2 + 2 * nr], S->ev[2] };
        for( int k = 0; k < 4; k++ )
            if( cudaEventElapsedTime( &S->stream_ms[k], S->copy_ev[0], marks[k] ) != cudaSuccess ) {
                cudaGetLastError(); // informative only
                S->stream_ms[k] = -1.0f;
            }
        // a spill re-laid the species out, or particles left: the ranges packed during the
        // step are not the new state
        if( valid && copied == n && S->h_flags[1 + species] == 0 && S->h_flags[1 + S->max_species + species] == 0 ) {
            std::memcpy( hout, &n, 8 );
            // the sums saw every particle unless some species spilled (its spilled
            // particles were in the overflow list)
            bool spill = false;
            for( size_t k = 0; k < S->sp.size(); k++ ) spill = spill || S->h_flags[1 + k] != 0;
            S->energy_valid = !spill;
            return SG_OK;
        }
    } else {
        r = finish_step( S, false );
        if( r ) return r;
    }
    r = sg_sim_pack_state( S, species, host_out );
    if( r ) return r;
    SG_CUDA_TRY( cudaStreamSynchronize( S->stream ) );
    return SG_OK;
}

int sg_sim_stream_timing( sg_sim *S, float *ms )
{
    SG_REQUIRE( S && ms, "NULL argument" );
    for( int k = 0; k < 4; k++ ) ms[k] = S->stream_ms[k];
    return SG_OK;
}

// E and the time-centred B_m (DiagnosticScalar.cpp:640-646), in that order.
static Norm2Set energy_fields( const sg_sim *S )
{
    Norm2Set f{};
    const int comps[6] = { 0, 1, 2, 6, 7, 8 };
    for( int k = 0; k < 6; k++ ) {
        const int c = comps[k];
        f.a[k] = S->fptr[c];
        f.e1[k] = ext( S->g, 1, comp_stag( c, 1 ) );
        f.e2[k] = ext( S->g, 2, comp_stag( c, 2 ) );
    }
    return f;
}

// Enqueues the energy sums on st into S->h_energy: each species' sum of w (gamma - 1)
// over buffer `cur ^ next` (next: the buffers a step enqueued just before writes) and
// the squared E and time-centred B_m.
int enqueue_energy( sg_sim *S, cudaStream_t st, bool next )
{
    SG_CUDA_TRY( cudaMemsetAsync( S->d_red, 0, 16 * sizeof( double ), st ) );
    const int nt = S->g.ntiles;
    for( size_t k = 0; k < S->sp.size(); k++ ) {
        SpeciesState &s = S->sp[k];
        const int b = next ? 1 - s.cur : s.cur;
        if( S->mixed ) k_kinetic<true><<<std::min( nt, 1216 ), 256, 0, st>>>( nt, s.seg_start, s.count[b], s.bm[b], S->d_red + 2 + k % 14 );
        else k_kinetic<false><<<std::min( nt, 1216 ), 256, 0, st>>>( nt, s.seg_start, s.count[b], s.bd[b], S->d_red + 2 + k % 14 );
        SG_LAUNCH_CHECK( "k_kinetic" );
    }
    const Norm2Set f = energy_fields( S );
    if( S->mixed ) k_norm2<float><<<dim3( 304, 6 ), 256, 0, st>>>( S->g, f, 0, S->d_red + 1 );
    else k_norm2<double><<<dim3( 304, 6 ), 256, 0, st>>>( S->g, f, 0, S->d_red + 1 );
    SG_LAUNCH_CHECK( "k_norm2" );
    SG_CUDA_TRY( cudaMemcpyAsync( S->h_energy, S->d_red, 16 * sizeof( double ), cudaMemcpyDeviceToHost, st ) );
    return SG_OK;
}

int sg_sim_energy( sg_sim *S, double *ukin, double *uelm )
{
    SG_REQUIRE( S, "NULL simulation" );
    // a streamed step leaves the sums of the state it produced
    if( !S->energy_valid ) {
        int r = enqueue_energy( S, S->stream, false );
        if( r ) return r;
    }
    SG_CUDA_TRY( cudaStreamSynchronize( S->stream ) );
    const double *h = S->h_energy;
    double vol = 1.0;
    for( int d = 0; d < S->g.ndim; d++ ) vol *= S->g.dx[d];
    double uk = 0.0;
    for( size_t k = 0; k < S->sp.size(); k++ ) uk += S->sp[k].mass * h[2 + k % 14];
    if( ukin ) *ukin = uk;
    if( uelm ) *uelm = 0.5 * vol * h[1];
    return SG_OK;
}

int sg_sim_species_scalars( sg_sim *S, int species, double *out )
{
    SG_REQUIRE( S && out, "NULL argument" );
    SG_REQUIRE( species >= 0 && species < ( int )S->sp.size(), "no species %d", species );
    SpeciesState &s = S->sp[species];
    cudaStream_t st = S->stream;
    const int nt = S->g.ntiles;
    SG_CUDA_TRY( cudaMemsetAsync( S->d_red, 0, 2 * sizeof( double ), st ) );
    if( S->mixed ) k_species_sums<true><<<std::min( nt, 1216 ), 256, 0, st>>>( nt, s.seg_start, s.count[s.cur], s.bm[s.cur], S->d_red );
    else k_species_sums<false><<<std::min( nt, 1216 ), 256, 0, st>>>( nt, s.seg_start, s.count[s.cur], s.bd[s.cur], S->d_red );
    SG_LAUNCH_CHECK( "k_species_sums" );
    double h[2];
    SG_CUDA_TRY( cudaMemcpyAsync( h, S->d_red, sizeof( h ), cudaMemcpyDeviceToHost, st ) );
    SG_CUDA_TRY( cudaStreamSynchronize( st ) );
    out[0] = h[0];
    out[1] = ( double )s.npart;
    out[2] = s.charge * h[0];
    out[3] = s.mass * h[1];
    return SG_OK;
}

int sg_sim_field_energies( sg_sim *S, double *out )
{
    SG_REQUIRE( S && out, "NULL argument" );
    cudaStream_t st = S->stream;
    SG_CUDA_TRY( cudaMemsetAsync( S->d_red, 0, 6 * sizeof( double ), st ) );
    const Norm2Set f = energy_fields( S );
    if( S->mixed ) k_norm2<float><<<dim3( 304, 6 ), 256, 0, st>>>( S->g, f, 1, S->d_red );
    else k_norm2<double><<<dim3( 304, 6 ), 256, 0, st>>>( S->g, f, 1, S->d_red );
    SG_LAUNCH_CHECK( "k_norm2" );
    double h[6];
    SG_CUDA_TRY( cudaMemcpyAsync( h, S->d_red, sizeof( h ), cudaMemcpyDeviceToHost, st ) );
    SG_CUDA_TRY( cudaStreamSynchronize( st ) );
    double vol = 1.0;
    for( int d = 0; d < S->g.ndim; d++ ) vol *= S->g.dx[d];
    for( int k = 0; k < 6; k++ ) out[k] = 0.5 * vol * h[k];
    return SG_OK;
}

} // extern "C"

// ==============================================================================
// Charge density, initial-field Poisson solve (FP64 conjugate gradient) and
// the charge-conservation residual.
// ==============================================================================
namespace sg {
namespace {

// rho of the current particle positions (Projector3D2Order::basic, type 0,
// src/Projector/Projector3D2Order.cpp:526-618), FP64 accumulation in a
// per-tile shared array, flushed into the FP64 rho array (reference layout,
// primal, ghosts).  One block per tile.
template <int DIM, bool MIXED>
__global__ void k_rho_tiles( GridInfo g, const int64_t *__restrict__ seg_start, const int *__restrict__ count,
                             PBuf<MIXED> b, double cw, double *__restrict__ rho )
{
    extern __shared__ __align__( 16 ) unsigned char smem_raw[];
    double *sR = reinterpret_cast<double *>( smem_raw );
    const TileDims td = tile_dims( g );
    const int jsz = td.JX * td.JY * td.JZ;
    const int tile = blockIdx.x;
    int tz = 0, ty, tx;
    if( DIM == 3 ) {
        tz = tile % g.nt[2];
        ty = ( tile / g.nt[2] ) % g.nt[1];
        tx = tile / ( g.nt[2] * g.nt[1] );
    } else {
        ty = tile % g.nt[1];
        tx = tile / g.nt[1];
    }
    const int i0[3] = { tx * g.T[0], ty * g.T[1], DIM == 3 ? tz * g.T[2] : 0 };
    for( int e = threadIdx.x; e < jsz; e += blockDim.x ) sR[e] = 0.0;
    __syncthreads();
    const int n = count[tile];
    const int64_t s0 = seg_start[tile];
    for( int q = threadIdx.x; q < n; q += blockDim.x ) {
        const int64_t src = s0 + q;
        int node[3] = { 0, 0, 0 };
        double dl[3] = { 0.0, 0.0, 0.0 };
        if constexpr( MIXED ) {
            unpack_key( DIM, b.key[src], node[0], node[1], node[2] );
            for( int d = 0; d < DIM; d++ ) dl[d] = ( double )b.d[d][src];
        } else {
            for( int d = 0; d < DIM; d++ ) {
                double xn = b.x[d][src] * g.dxi[d];
                int ip = round_half_away( xn );
                if( ip >= g.N[d] ) { ip -= g.N[d]; xn -= ( double )g.N[d]; }
                node[d] = ip;
                dl[d] = xn - ( double )ip;
            }
        }
        double S[3][3];
        int l[3] = { 0, 0, 0 };
        bool inside = true;
        for( int d = 0; d < 3; d++ ) {
            if( d < DIM ) {
                bspline2( dl[d], S[d][0], S[d][1], S[d][2] );
                l[d] = node[d] - i0[d];
                if( l[d] < 0 || l[d] >= g.T[d] ) inside = false;
            } else {
                S[d][0] = S[d][2] = 0.0;
                S[d][1] = 1.0;
            }
        }
        if( !inside ) continue; // cannot happen for a sorted buffer
        const double c = cw * ( double )b.w[src];
        // nodes node-1 .. node+1 -> tile index l+1 .. l+3 (tile origin at node i0-2)
        for( int a = 0; a < 3; a++ )
            for( int bb = 0; bb < 3; bb++ )
                for( int cc = 0; cc < ( DIM == 3 ? 3 : 1 ); cc++ ) {
                    const double v = c * S[0][a] * S[1][bb] * ( DIM == 3 ? S[2][cc] : 1.0 );
                    const int iz = DIM == 3 ? l[2] + 1 + cc : 0;
                    atomicAdd( &sR[( ( l[0] + 1 + a ) * td.JY + ( l[1] + 1 + bb ) ) * td.JZ + iz], v );
                }
    }
    __syncthreads();
    const int nx = ext( g, 0, 0 ), ny = ext( g, 1, 0 ), nz = ext( g, 2, 0 );
    for( int e = threadIdx.x; e < jsz; e += blockDim.x ) {
        const double v = sR[e];
        if( v == 0.0 ) continue;
        const int cz = e % td.JZ, cy = ( e / td.JZ ) % td.JY, cx = e / ( td.JZ * td.JY );
        const int gx = i0[0] + OS - 2 + cx, gy = i0[1] + OS - 2 + cy, gz = DIM == 3 ? i0[2] + OS - 2 + cz : 0;
        if( gx < nx && gy < ny && gz < nz ) atomicAdd( &rho[( ( int64_t )gx * ny + gy ) * nz + gz], v );
    }
}

// Periodic fold of one primal array (as k_fold, for rho).
__global__ void k_fold_one( GridInfo g, int d, double *a )
{
    const int e0 = ext( g, 0, 0 ), e1 = ext( g, 1, 0 ), e2 = ext( g, 2, 0 );
    int se[3] = { e0, e1, e2 };
    se[d] = 1 + 2 * OS;
    const int64_t n = ( int64_t )se[0] * se[1] * se[2];
    for( int64_t t = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x; t < n; t += ( int64_t )gridDim.x * blockDim.x ) {
        const int k = ( int )( t % se[2] ), j = ( int )( ( t / se[2] ) % se[1] ), i = ( int )( t / ( ( int64_t )se[2] * se[1] ) );
        int i2 = i, j2 = j, k2 = k;
        if( d == 0 ) i2 += g.N[0]; else if( d == 1 ) j2 += g.N[1]; else k2 += g.N[2];
        const int64_t a1 = ( ( int64_t )i * e1 + j ) * e2 + k, a2 = ( ( int64_t )i2 * e1 + j2 ) * e2 + k2;
        const double v = a[a2] + a[a1];
        a[a2] = v;
        a[a1] = v;
    }
}

// Physical node t (x-major over N^ndim) <-> array index of the ghosted array.
__device__ __forceinline__ void phys_ijk( const GridInfo &g, int64_t t, int &i, int &j, int &k )
{
    const int n1 = g.N[1], n2 = g.ndim == 3 ? g.N[2] : 1;
    k = ( int )( t % n2 );
    j = ( int )( ( t / n2 ) % n1 );
    i = ( int )( t / ( ( int64_t )n2 * n1 ) );
}

__device__ __forceinline__ int64_t phys_lin( const GridInfo &g, int i, int j, int k )
{
    const int n1 = g.N[1], n2 = g.ndim == 3 ? g.N[2] : 1;
    return ( ( int64_t )i * n1 + j ) * n2 + k;
}

__device__ __forceinline__ int wrapi( int i, int n ) { return i < 0 ? i + n : ( i >= n ? i - n : i ); }

// b = rho (physical nodes) minus the mean given in mean[0]; r = -b... the CG
// starts from phi = 0, r = -rho, p = r (ElectroMagn3D::initPoisson).
__global__ void k_cg_init( GridInfo g, const double *__restrict__ rho_g, const double *__restrict__ sums,
                           double *__restrict__ phi, double *__restrict__ r, double *__restrict__ p, int64_t n )
{
    const double mean = sums[0] / ( double )n;
    for( int64_t t = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x; t < n; t += ( int64_t )gridDim.x * blockDim.x ) {
        int i, j, k;
        phys_ijk( g, t, i, j, k );
        const int ny = ext( g, 1, 0 ), nz = ext( g, 2, 0 );
        const double v = rho_g[( ( int64_t )( i + OS ) * ny + ( j + OS ) ) * nz + ( g.ndim == 3 ? k + OS : 0 )] - mean;
        phi[t] = 0.0;
        r[t] = -v;
        p[t] = -v;
    }
}

// sum of rho over the physical nodes (for the mean) -> sums[0]
__global__ void k_rho_sum( GridInfo g, const double *__restrict__ rho_g, int64_t n, double *__restrict__ sums )
{
    double acc = 0.0;
    for( int64_t t = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x; t < n; t += ( int64_t )gridDim.x * blockDim.x ) {
        int i, j, k;
        phys_ijk( g, t, i, j, k );
        const int ny = ext( g, 1, 0 ), nz = ext( g, 2, 0 );
        acc += rho_g[( ( int64_t )( i + OS ) * ny + ( j + OS ) ) * nz + ( g.ndim == 3 ? k + OS : 0 )];
    }
    acc = block_sum( acc );
    if( threadIdx.x == 0 ) atomicAdd( sums, acc );
}

__global__ void k_dot( const double *__restrict__ a, const double *__restrict__ b, int64_t n, double *__restrict__ out )
{
    double acc = 0.0;
    for( int64_t t = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x; t < n; t += ( int64_t )gridDim.x * blockDim.x )
        acc += a[t] * b[t];
    acc = block_sum( acc );
    if( threadIdx.x == 0 ) atomicAdd( out, acc );
}

// Ap = periodic 7-point (5-point in 2D) Laplacian of p (ElectroMagn3D::compute_Ap), and p.Ap -> s[1]
__global__ void k_cg_ap( GridInfo g, const double *__restrict__ p, double *__restrict__ Ap, int64_t n,
                         double *__restrict__ s )
{
    const double ix2 = g.dxi[0] * g.dxi[0], iy2 = g.dxi[1] * g.dxi[1];
    const double iz2 = g.ndim == 3 ? g.dxi[2] * g.dxi[2] : 0.0;
    const double two = 2.0 * ( ix2 + iy2 + iz2 );
    double acc = 0.0;
    for( int64_t t = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x; t < n; t += ( int64_t )gridDim.x * blockDim.x ) {
        int i, j, k;
        phys_ijk( g, t, i, j, k );
        double v = ix2 * ( p[phys_lin( g, wrapi( i - 1, g.N[0] ), j, k )] + p[phys_lin( g, wrapi( i + 1, g.N[0] ), j, k )] )
                   + iy2 * ( p[phys_lin( g, i, wrapi( j - 1, g.N[1] ), k )] + p[phys_lin( g, i, wrapi( j + 1, g.N[1] ), k )] );
        if( g.ndim == 3 ) v += iz2 * ( p[phys_lin( g, i, j, wrapi( k - 1, g.N[2] ) )] + p[phys_lin( g, i, j, wrapi( k + 1, g.N[2] ) )] );
        v -= two * p[t];
        Ap[t] = v;
        acc += p[t] * v;
    }
    acc = block_sum( acc );
    if( threadIdx.x == 0 ) atomicAdd( &s[1], acc );
}

// alpha = r.r / p.Ap; phi += alpha p; r -= alpha Ap; r_new.r_new -> s[2] (update_pand_r)
__global__ void k_cg_update_r( const double *__restrict__ p, const double *__restrict__ Ap, double *__restrict__ phi,
                               double *__restrict__ r, int64_t n, double *__restrict__ s )
{
    const double alpha = s[0] / s[1];
    double acc = 0.0;
    for( int64_t t = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x; t < n; t += ( int64_t )gridDim.x * blockDim.x ) {
        phi[t] += alpha * p[t];
        const double rv = r[t] - alpha * Ap[t];
        r[t] = rv;
        acc += rv * rv;
    }
    acc = block_sum( acc );
    if( threadIdx.x == 0 ) atomicAdd( &s[2], acc );
}

// p = r + beta p with beta = r_new.r_new / r.r (update_p)
__global__ void k_cg_update_p( const double *__restrict__ r, double *__restrict__ p, int64_t n,
                               const double *__restrict__ s )
{
    const double beta = s[2] / s[0];
    for( int64_t t = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x; t < n; t += ( int64_t )gridDim.x * blockDim.x )
        p[t] = r[t] + beta * p[t];
}

// s[0] <- s[2], s[1] = s[2] = 0, s[3] = ctrl = r.r / n
__global__ void k_cg_scalars( double *s, int64_t n )
{
    s[0] = s[2];
    s[1] = 0.0;
    s[2] = 0.0;
    s[3] = s[0] / ( double )n;
}

// E_d on the dual nodes from phi (ElectroMagn3D::initE): E_d(i) = (phi(i-1) - phi(i)) / dx_d,
// physical layout; also accumulates each component's sum (for the mean) into sums[d].
__global__ void k_efield( GridInfo g, const double *__restrict__ phi, double *__restrict__ E, int64_t n,
                          double *__restrict__ sums )
{
    const int d = blockIdx.y;
    double acc = 0.0;
    for( int64_t t = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x; t < n; t += ( int64_t )gridDim.x * blockDim.x ) {
        int i, j, k;
        phys_ijk( g, t, i, j, k );
        int a = i, b = j, c = k;
        if( d == 0 ) a = wrapi( i - 1, g.N[0] );
        else if( d == 1 ) b = wrapi( j - 1, g.N[1] );
        else c = wrapi( k - 1, g.N[2] );
        const double v = ( phi[phys_lin( g, a, b, c )] - phi[t] ) * g.dxi[d];
        E[( int64_t )d * n + t] = v;
        acc += v;
    }
    acc = block_sum( acc );
    if( threadIdx.x == 0 ) atomicAdd( &sums[d], acc );
}

// Writes E_d minus its mean into every point (ghosts included) of the simulation's E_d array.
template <class T>
__global__ void k_efield_store( GridInfo g, const double *__restrict__ E, int64_t n, const double *__restrict__ sums,
                                T *__restrict__ dst, int d )
{
    const int sx = stag( d, 0 ), sy = stag( d, 1 ), sz = stag( d, 2 );
    const int e0 = ext( g, 0, sx ), e1 = ext( g, 1, sy ), e2 = ext( g, 2, sz );
    const int64_t tot = ( int64_t )e0 * e1 * e2;
    const double mean = sums[d] / ( double )n;
    for( int64_t t = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += ( int64_t )gridDim.x * blockDim.x ) {
        const int k = ( int )( t % e2 ), j = ( int )( ( t / e2 ) % e1 ), i = ( int )( t / ( ( int64_t )e2 * e1 ) );
        const int pi = ( ( i - OS ) % g.N[0] + g.N[0] ) % g.N[0];
        const int pj = ( ( j - OS ) % g.N[1] + g.N[1] ) % g.N[1];
        const int pk = g.ndim == 3 ? ( ( k - OS ) % g.N[2] + g.N[2] ) % g.N[2] : 0;
        dst[t] = ( T )( E[( int64_t )d * n + phys_lin( g, pi, pj, pk )] - mean );
    }
}

// max |div E - (rho - mean rho)| and max |rho - mean rho| over the physical nodes -> out[0], out[1]
// (as unsigned-long-long bit patterns of non-negative doubles, so atomicMax orders them).
template <class T>
__global__ void k_residual( GridInfo g, const T *__restrict__ Ex, const T *__restrict__ Ey, const T *__restrict__ Ez,
                            const T *__restrict__ Cx, const T *__restrict__ Cy, const T *__restrict__ Cz,
                            const double *__restrict__ rho_g, const double *__restrict__ sums, int64_t n,
                            unsigned long long *__restrict__ out )
{
    // the mixed form's E is the pair E - C (C: compensation of the Ampere updates)
    auto ev = []( const T *E, const T *C, int64_t i ) { return C ? ( double )E[i] - ( double )C[i] : ( double )E[i]; };
    const double mean = sums[0] / ( double )n;
    const int nyp = ext( g, 1, 0 ), nzp = ext( g, 2, 0 );
    double m0 = 0.0, m1 = 0.0;
    for( int64_t t = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x; t < n; t += ( int64_t )gridDim.x * blockDim.x ) {
        int i, j, k;
        phys_ijk( g, t, i, j, k );
        const int a = i + OS, b = j + OS, c = g.ndim == 3 ? k + OS : 0;
        // primal node (a,b,c): Ex dual in x at a and a+1, etc.
        double div = ( ev( Ex, Cx, ( ( int64_t )( a + 1 ) * nyp + b ) * nzp + c ) - ev( Ex, Cx, ( ( int64_t )a * nyp + b ) * nzp + c ) ) * g.dxi[0]
                     + ( ev( Ey, Cy, ( ( int64_t )a * ( nyp + 1 ) + b + 1 ) * nzp + c ) - ev( Ey, Cy, ( ( int64_t )a * ( nyp + 1 ) + b ) * nzp + c ) ) * g.dxi[1];
        if( g.ndim == 3 )
            div += ( ev( Ez, Cz, ( ( int64_t )a * nyp + b ) * ( nzp + 1 ) + c + 1 ) - ev( Ez, Cz, ( ( int64_t )a * nyp + b ) * ( nzp + 1 ) + c ) ) * g.dxi[2];
        const double rv = rho_g[( ( int64_t )a * nyp + b ) * nzp + c] - mean;
        m0 = fmax( m0, fabs( div - rv ) );
        m1 = fmax( m1, fabs( rv ) );
    }
    for( int o = 16; o > 0; o >>= 1 ) {
        m0 = fmax( m0, __shfl_down_sync( 0xffffffffu, m0, o ) );
        m1 = fmax( m1, __shfl_down_sync( 0xffffffffu, m1, o ) );
    }
    if( ( threadIdx.x & 31 ) == 0 ) {
        atomicMax( &out[0], ( unsigned long long )__double_as_longlong( m0 ) );
        atomicMax( &out[1], ( unsigned long long )__double_as_longlong( m1 ) );
    }
}

// Deposits rho of all species (FP64) into S->rho (reference layout, primal), folded.
int deposit_rho( sg_sim *S, double *rho )
{
    cudaStream_t st = S->stream;
    const GridInfo &g = S->g;
    SG_CUDA_TRY( cudaMemsetAsync( rho, 0, ( size_t )ext( g, 0, 0 ) * ext( g, 1, 0 ) * ext( g, 2, 0 ) * sizeof( double ), st ) );
    const TileDims td = tile_dims( g );
    const size_t smem = ( size_t )td.JX * td.JY * td.JZ * sizeof( double );
    double vol = 1.0;
    for( int d = 0; d < g.ndim; d++ ) vol *= g.dx[d];
    for( auto &s : S->sp ) {
        const double cw = s.charge / vol;
        if( g.ndim == 3 ) {
            if( S->mixed ) k_rho_tiles<3, true><<<g.ntiles, 128, smem, st>>>( g, s.seg_start, s.count[s.cur], s.bm[s.cur], cw, rho );
            else k_rho_tiles<3, false><<<g.ntiles, 128, smem, st>>>( g, s.seg_start, s.count[s.cur], s.bd[s.cur], cw, rho );
        } else {
            if( S->mixed ) k_rho_tiles<2, true><<<g.ntiles, 128, smem, st>>>( g, s.seg_start, s.count[s.cur], s.bm[s.cur], cw, rho );
            else k_rho_tiles<2, false><<<g.ntiles, 128, smem, st>>>( g, s.seg_start, s.count[s.cur], s.bd[s.cur], cw, rho );
        }
        SG_LAUNCH_CHECK( "k_rho_tiles" );
    }
    for( int d = 0; d < g.ndim; d++ ) {
        k_fold_one<<<1024, 256, 0, st>>>( g, d, rho );
        SG_LAUNCH_CHECK( "k_fold_one" );
    }
    return SG_OK;
}

int64_t phys_nodes( const GridInfo &g )
{
    int64_t n = 1;
    for( int d = 0; d < g.ndim; d++ ) n *= g.N[d];
    return n;
}

} // namespace
} // namespace sg

extern "C" {

int sg_sim_get_rho( sg_sim *S, double *host )
{
    SG_REQUIRE( S && host, "NULL argument" );
    SG_REQUIRE( !S->g.open[0] && !S->g.open[1] && !S->g.open[2], "charge density, Poisson and residual need a periodic grid" );
    const GridInfo &g = S->g;
    const size_t n = ( size_t )ext( g, 0, 0 ) * ext( g, 1, 0 ) * ext( g, 2, 0 );
    double *rho = nullptr;
    SG_CUDA_TRY( cudaMallocAsync( &rho, n * sizeof( double ), S->stream ) );
    int r = deposit_rho( S, rho );
    if( r == SG_OK ) {
        SG_CUDA_TRY( cudaMemcpyAsync( host, rho, n * sizeof( double ), cudaMemcpyDeviceToHost, S->stream ) );
    }
    release_async( rho, S->stream );
    SG_CUDA_TRY( cudaStreamSynchronize( S->stream ) );
    return r;
}

int sg_sim_solve_poisson( sg_sim *S, double max_error, int max_iter, int *iterations, double *ctrl_out )
{
    if( S ) S->energy_valid = false;
    SG_REQUIRE( S, "NULL simulation" );
    SG_REQUIRE( !S->g.open[0] && !S->g.open[1] && !S->g.open[2], "charge density, Poisson and residual need a periodic grid" );
    SG_REQUIRE( max_iter >= 0, "max_iter < 0" );
    const GridInfo &g = S->g;
    cudaStream_t st = S->stream;
    S->pad_dirty = true; // E is replaced
    const int64_t n = phys_nodes( g );
    const size_t nrho = ( size_t )ext( g, 0, 0 ) * ext( g, 1, 0 ) * ext( g, 2, 0 );
    // scratch: rho (ghosted) + phi, r, p, Ap (physical) + E (ndim x physical) + scalars
    double *mem = nullptr;
    const size_t elems = nrho + ( 4 + ( size_t )g.ndim ) * ( size_t )n + 16;
    SG_CUDA_TRY( cudaMallocAsync( &mem, elems * sizeof( double ), st ) );
    double *rho = mem, *phi = rho + nrho, *r = phi + n, *p = r + n, *Ap = p + n, *E = Ap + n;
    double *s = E + ( size_t )g.ndim * n; // [0] r.r [1] p.Ap [2] rnew [3] ctrl [4] rho sum [8..10] E sums
    int rc = SG_OK;
    int it = 0;
    double ctrl = 0.0;
    do {
        if( cudaMemsetAsync( s, 0, 16 * sizeof( double ), st ) != cudaSuccess ) { rc = set_error( SG_ERR_CUDA, "memset" ); break; }
        if( ( rc = deposit_rho( S, rho ) ) ) break;
        k_rho_sum<<<1024, 256, 0, st>>>( g, rho, n, s + 4 );
        k_cg_init<<<1024, 256, 0, st>>>( g, rho, s + 4, phi, r, p, n );
        k_dot<<<1024, 256, 0, st>>>( r, r, n, s + 2 );
        k_cg_scalars<<<1, 1, 0, st>>>( s, n );
        if( cudaGetLastError() != cudaSuccess ) { rc = set_error( SG_ERR_CUDA, "CG init launch failed" ); break; }
        double h[4];
        if( cudaMemcpyAsync( h, s, 4 * sizeof( double ), cudaMemcpyDeviceToHost, st ) != cudaSuccess ||
            cudaStreamSynchronize( st ) != cudaSuccess ) { rc = set_error( SG_ERR_CUDA, "CG init failed" ); break; }
        ctrl = h[3];
        const int check_every = 16;
        while( ctrl > max_error && it < max_iter ) {
            const int todo = std::min( check_every, max_iter - it );
            for( int k = 0; k < todo; k++ ) {
                k_cg_ap<<<1216, 256, 0, st>>>( g, p, Ap, n, s );
                k_cg_update_r<<<1216, 256, 0, st>>>( p, Ap, phi, r, n, s );
                k_cg_update_p<<<1216, 256, 0, st>>>( r, p, n, s );
                k_cg_scalars<<<1, 1, 0, st>>>( s, n );
            }
            if( cudaGetLastError() != cudaSuccess ) { rc = set_error( SG_ERR_CUDA, "CG launch failed" ); break; }
            if( cudaMemcpyAsync( h, s, 4 * sizeof( double ), cudaMemcpyDeviceToHost, st ) != cudaSuccess ||
                cudaStreamSynchronize( st ) != cudaSuccess ) { rc = set_error( SG_ERR_CUDA, "CG iteration failed" ); break; }
            // iterations past convergence inside a batch only shrink r further; count them all
            it += todo;
            ctrl = h[3];
        }
        if( rc ) break;
        dim3 ge( 1024, g.ndim );
        k_efield<<<ge, 256, 0, st>>>( g, phi, E, n, s + 8 );
        for( int d = 0; d < g.ndim; d++ ) {
            if( S->mixed ) k_efield_store<float><<<1024, 256, 0, st>>>( g, E, n, s + 8, static_cast<float *>( S->fptr[d] ), d );
            if( S->ecomp[d] ) cudaMemsetAsync( S->ecomp[d], 0, S->fsize[d] * S->esz, st );
            else k_efield_store<double><<<1024, 256, 0, st>>>( g, E, n, s + 8, static_cast<double *>( S->fptr[d] ), d );
        }
        if( cudaGetLastError() != cudaSuccess ) { rc = set_error( SG_ERR_CUDA, "E from phi failed" ); break; }
    } while( 0 );
    release_async( mem, st );
    if( cudaStreamSynchronize( st ) != cudaSuccess && rc == SG_OK ) rc = set_error( SG_ERR_CUDA, "Poisson solve failed" );
    if( iterations ) *iterations = it;
    if( ctrl_out ) *ctrl_out = ctrl;
    drop_graphs( S );
    return rc;
}

int sg_sim_charge_residual( sg_sim *S, double *residual, double *rho_max )
{
    SG_REQUIRE( S && residual, "NULL argument" );
    SG_REQUIRE( !S->g.open[0] && !S->g.open[1] && !S->g.open[2], "charge density, Poisson and residual need a periodic grid" );
    const GridInfo &g = S->g;
    cudaStream_t st = S->stream;
    const int64_t n = phys_nodes( g );
    const size_t nrho = ( size_t )ext( g, 0, 0 ) * ext( g, 1, 0 ) * ext( g, 2, 0 );
    double *mem = nullptr;
    SG_CUDA_TRY( cudaMallocAsync( &mem, ( nrho + 8 ) * sizeof( double ), st ) );
    double *rho = mem, *s = mem + nrho;
    unsigned long long *mx = reinterpret_cast<unsigned long long *>( s + 4 );
    int rc = SG_OK;
    do {
        if( cudaMemsetAsync( s, 0, 8 * sizeof( double ), st ) != cudaSuccess ) { rc = set_error( SG_ERR_CUDA, "memset" ); break; }
        if( ( rc = deposit_rho( S, rho ) ) ) break;
        k_rho_sum<<<1024, 256, 0, st>>>( g, rho, n, s );
        if( S->mixed )
            k_residual<float><<<1024, 256, 0, st>>>( g, static_cast<float *>( S->fptr[0] ), static_cast<float *>( S->fptr[1] ), static_cast<float *>( S->fptr[2] ),
                                                      static_cast<float *>( S->ecomp[0] ), static_cast<float *>( S->ecomp[1] ), static_cast<float *>( S->ecomp[2] ), rho, s, n, mx );
        else
            k_residual<double><<<1024, 256, 0, st>>>( g, static_cast<double *>( S->fptr[0] ), static_cast<double *>( S->fptr[1] ), static_cast<double *>( S->fptr[2] ),
                                                       nullptr, nullptr, nullptr, rho, s, n, mx );
        if( cudaGetLastError() != cudaSuccess ) { rc = set_error( SG_ERR_CUDA, "residual launch failed" ); break; }
    } while( 0 );
    unsigned long long h[2] = { 0, 0 };
    if( rc == SG_OK ) cudaMemcpyAsync( h, mx, sizeof( h ), cudaMemcpyDeviceToHost, st );
    release_async( mem, st );
    if( cudaStreamSynchronize( st ) != cudaSuccess && rc == SG_OK ) rc = set_error( SG_ERR_CUDA, "residual failed" );
    if( rc ) return rc;
    double m0, m1;
    std::memcpy( &m0, &h[0], 8 );
    std::memcpy( &m1, &h[1], 8 );
    *residual = m1 > 0.0 ? m0 / m1 : m0;
    if( rho_max ) *rho_max = m1;
    return SG_OK;
}

} // extern "C"
