// Drop-in FP64 operators on one patch's arrays (the reference's layout).
//
// These are the entry points a reference operator class would call in place
// of its CPU loop: gather (Interpolator), push (Pusher), Esirkepov deposit
// (Projector), Yee Ampere/Faraday (Solver) and the B_m save/centre.  They work
// on caller-owned device arrays with ghost cells and an arbitrary patch origin,
// one thread per particle or per grid point.  The fused, tiled timestep of the
// simulation object (sim.cu) is the performance path; these kernels are the
// per-operator interface and are held to the same FP64 parity.

#include "common.cuh"

#include <cstring>
#include <mutex>

namespace sg {

namespace {

thread_local std::string g_last_error;

// Set by an operator kernel that met a particle whose stencil leaves the
// patch arrays (the access is clamped inside the arrays and the particle's
// result is meaningless); reported and cleared by the next
// sg_project_currents call, which synchronises.
__device__ int g_bounds_flag = 0;

struct Dims {
    int ndim;
    int nxp, nyp, nzp; // primal extents (nzp = 1 in 2D)
    int db[3];
    double dxi[3];
};

Dims make_dims( const sg_grid_geom *g )
{
    Dims d{};
    d.ndim = g->ndim;
    d.nxp = g->n_prim[0];
    d.nyp = g->n_prim[1];
    d.nzp = g->ndim == 3 ? g->n_prim[2] : 1;
    for( int k = 0; k < 3; k++ ) {
        d.db[k] = k < g->ndim ? g->domain_begin[k] : 0;
        d.dxi[k] = k < g->ndim ? 1.0 / g->cell_length[k] : 0.0;
    }
    return d;
}

__device__ __forceinline__ int64_t lin( int i, int j, int k, int ny, int nz )
{
    return ( ( int64_t )i * ny + j ) * nz + k;
}

// ---- gather -----------------------------------------------------------------
__device__ __forceinline__ double g3( const double *__restrict__ f, const double *cx, const double *cy,
                                      const double *cz, int i, int j, int k, int ny, int nz )
{
    double r = 0.0;
#pragma unroll
    for( int a = 0; a < 3; a++ )
#pragma unroll
        for( int b = 0; b < 3; b++ )
#pragma unroll
            for( int c = 0; c < 3; c++ ) r += cx[a] * cy[b] * cz[c] * __ldg( &f[lin( i + a - 1, j + b - 1, k + c - 1, ny, nz )] );
    return r;
}

__device__ __forceinline__ double g2( const double *__restrict__ f, const double *cx, const double *cy, int i, int j,
                                      int ny )
{
    double r = 0.0;
#pragma unroll
    for( int a = 0; a < 3; a++ )
#pragma unroll
        for( int b = 0; b < 3; b++ ) r += cx[a] * cy[b] * __ldg( &f[( int64_t )( i + a - 1 ) * ny + ( j + b - 1 )] );
    return r;
}

template <int DIM>
__global__ void k_interpolate( Dims d, const double *__restrict__ Ex, const double *__restrict__ Ey,
                               const double *__restrict__ Ez, const double *__restrict__ Bx,
                               const double *__restrict__ By, const double *__restrict__ Bz, int64_t n,
                               const double *__restrict__ pos, double *__restrict__ Epart,
                               double *__restrict__ Bpart, int *__restrict__ iold, double *__restrict__ delta )
{
    const int64_t p = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x;
    if( p >= n ) return;
    int ip[3], id[3];
    double cp[3][3], cd[3][3], dp[3];
#pragma unroll
    for( int k = 0; k < DIM; k++ ) {
        const double xn = pos[k * n + p] * d.dxi[k];
        ip[k] = round_half_away( xn );
        dp[k] = xn - ( double )ip[k];
        bspline2( dp[k], cp[k][0], cp[k][1], cp[k][2] );
        id[k] = round_half_away( xn + 0.5 );
        bspline2( xn - ( double )id[k] + 0.5, cd[k][0], cd[k][1], cd[k][2] );
        ip[k] -= d.db[k];
        id[k] -= d.db[k];
        const int np = k == 0 ? d.nxp : ( k == 1 ? d.nyp : d.nzp );
        if( ip[k] < 1 || ip[k] > np - 2 || id[k] < 1 || id[k] > np - 1 ) {
            atomicExch( &g_bounds_flag, 1 );
            ip[k] = min( max( ip[k], 1 ), np - 2 );
            id[k] = min( max( id[k], 1 ), np - 1 );
        }
    }
    const int nyd = d.nyp + 1, nzd = d.nzp + 1;
    if( DIM == 3 ) {
        Epart[p] = g3( Ex, cd[0], cp[1], cp[2], id[0], ip[1], ip[2], d.nyp, d.nzp );
        Epart[n + p] = g3( Ey, cp[0], cd[1], cp[2], ip[0], id[1], ip[2], nyd, d.nzp );
        Epart[2 * n + p] = g3( Ez, cp[0], cp[1], cd[2], ip[0], ip[1], id[2], d.nyp, nzd );
        Bpart[p] = g3( Bx, cp[0], cd[1], cd[2], ip[0], id[1], id[2], nyd, nzd );
        Bpart[n + p] = g3( By, cd[0], cp[1], cd[2], id[0], ip[1], id[2], d.nyp, nzd );
        Bpart[2 * n + p] = g3( Bz, cd[0], cd[1], cp[2], id[0], id[1], ip[2], nyd, d.nzp );
    } else {
        Epart[p] = g2( Ex, cd[0], cp[1], id[0], ip[1], d.nyp );
        Epart[n + p] = g2( Ey, cp[0], cd[1], ip[0], id[1], nyd );
        Epart[2 * n + p] = g2( Ez, cp[0], cp[1], ip[0], ip[1], d.nyp );
        Bpart[p] = g2( Bx, cp[0], cd[1], ip[0], id[1], nyd );
        Bpart[n + p] = g2( By, cd[0], cp[1], id[0], ip[1], d.nyp );
        Bpart[2 * n + p] = g2( Bz, cd[0], cd[1], id[0], id[1], nyd );
    }
#pragma unroll
    for( int k = 0; k < DIM; k++ ) {
        iold[k * n + p] = ip[k];
        delta[k * n + p] = dp[k];
    }
}

// ---- push -------------------------------------------------------------------
// One particle of the Boris (PusherBoris.cpp:82-127), Vay (PusherVay.cpp:92-173)
// or Higuera-Cary (PusherHigueraCary.cpp:93-167) scheme.  Returns 1/gamma.
template <int KIND, class T>
__device__ __forceinline__ T push_one( T qm, T Ex, T Ey, T Ez, T Bx, T By, T Bz, T &px, T &py, T &pz )
{
    if( KIND == 0 ) {
        T pxsm = qm * Ex, pysm = qm * Ey, pzsm = qm * Ez;
        const T umx = px + pxsm, umy = py + pysm, umz = pz + pzsm;
        const T lg = qm / sqrt( T( 1 ) + umx * umx + umy * umy + umz * umz );
        const T Tx = lg * Bx, Ty = lg * By, Tz = lg * Bz;
        const T inv_det = T( 1 ) / ( T( 1 ) + Tx * Tx + Ty * Ty + Tz * Tz );
        pxsm += ( ( T( 1 ) + Tx * Tx - Ty * Ty - Tz * Tz ) * umx + T( 2 ) * ( Tx * Ty + Tz ) * umy + T( 2 ) * ( Tz * Tx - Ty ) * umz ) * inv_det;
        pysm += ( T( 2 ) * ( Tx * Ty - Tz ) * umx + ( T( 1 ) - Tx * Tx + Ty * Ty - Tz * Tz ) * umy + T( 2 ) * ( Ty * Tz + Tx ) * umz ) * inv_det;
        pzsm += ( T( 2 ) * ( Tz * Tx + Ty ) * umx + T( 2 ) * ( Ty * Tz - Tx ) * umy + ( T( 1 ) - Tx * Tx - Ty * Ty + Tz * Tz ) * umz ) * inv_det;
        px = pxsm; py = pysm; pz = pzsm;
        return T( 1 ) / sqrt( T( 1 ) + pxsm * pxsm + pysm * pysm + pzsm * pzsm );
    } else if( KIND == 1 ) {
        const T g0 = T( 1 ) / sqrt( T( 1 ) + px * px + py * py + pz * pz );
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
        alpha = T( 1 ) / sqrt( T( 0.5 ) * ( s + sqrt( s * s + T( 4 ) * ( T2 + us2 ) ) ) );
        Tx *= alpha; Ty *= alpha; Tz *= alpha;
        s = T( 1 ) / ( T( 1 ) + Tx * Tx + Ty * Ty + Tz * Tz );
        alpha = upx * Tx + upy * Ty + upz * Tz;
        px = s * ( upx + alpha * Tx + Tz * upy - Ty * upz );
        py = s * ( upy + alpha * Ty + Tx * upz - Tz * upx );
        pz = s * ( upz + alpha * Tz + Ty * upx - Tx * upy );
        return T( 1 ) / sqrt( T( 1 ) + px * px + py * py + pz * pz );
    } else {
        T pxsm = qm * Ex, pysm = qm * Ey, pzsm = qm * Ez;
        const T umx = px + pxsm, umy = py + pysm, umz = pz + pzsm;
        const T gfm2 = T( 1 ) + umx * umx + umy * umy + umz * umz;
        T Tx = qm * Bx, Ty = qm * By, Tz = qm * Bz;
        const T beta2 = Tx * Tx + Ty * Ty + Tz * Tz;
        const T Tum = Tx * umx + Ty * umy + Tz * umz;
        const T lg = T( 1 ) / sqrt( T( 0.5 ) * ( gfm2 - beta2 + sqrt( ( gfm2 - beta2 ) * ( gfm2 - beta2 ) + T( 4 ) * ( beta2 + Tum * Tum ) ) ) );
        Tx *= lg; Ty *= lg; Tz *= lg;
        const T Tx2 = Tx * Tx, Ty2 = Ty * Ty, Tz2 = Tz * Tz;
        const T TxTy = Tx * Ty, TyTz = Ty * Tz, TzTx = Tz * Tx;
        const T inv_det = T( 1 ) / ( T( 1 ) + Tx2 + Ty2 + Tz2 );
        const T upx = ( ( T( 1 ) + Tx2 - Ty2 - Tz2 ) * umx + T( 2 ) * ( TxTy + Tz ) * umy + T( 2 ) * ( TzTx - Ty ) * umz ) * inv_det;
        const T upy = ( T( 2 ) * ( TxTy - Tz ) * umx + ( T( 1 ) - Tx2 + Ty2 - Tz2 ) * umy + T( 2 ) * ( TyTz + Tx ) * umz ) * inv_det;
        const T upz = ( T( 2 ) * ( TzTx + Ty ) * umx + T( 2 ) * ( TyTz - Tx ) * umy + ( T( 1 ) - Tx2 - Ty2 + Tz2 ) * umz ) * inv_det;
        px = pxsm + upx; py = pysm + upy; pz = pzsm + upz;
        return T( 1 ) / sqrt( T( 1 ) + px * px + py * py + pz * pz );
    }
}

template <int KIND>
__global__ void k_push( int ndim, double dt, double one_over_mass, int64_t n, double *__restrict__ pos,
                        double *__restrict__ mom, const short *__restrict__ charge,
                        const double *__restrict__ Epart, const double *__restrict__ Bpart,
                        double *__restrict__ invgf )
{
    const int64_t p = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x;
    if( p >= n ) return;
    const double qm = ( double )charge[p] * one_over_mass * ( dt / 2.0 );
    double px = mom[p], py = mom[n + p], pz = mom[2 * n + p];
    const double g = push_one<KIND, double>( qm, Epart[p], Epart[n + p], Epart[2 * n + p], Bpart[p], Bpart[n + p],
                                             Bpart[2 * n + p], px, py, pz );
    invgf[p] = g;
    mom[p] = px;
    mom[n + p] = py;
    mom[2 * n + p] = pz;
    if( KIND == 0 ) {
        const double vdt = g * dt;
        pos[p] += px * vdt;
        if( ndim > 1 ) pos[n + p] += py * vdt;
        if( ndim > 2 ) pos[2 * n + p] += pz * vdt;
    } else {
        pos[p] += dt * px * g;
        if( ndim > 1 ) pos[n + p] += dt * py * g;
        if( ndim > 2 ) pos[2 * n + p] += dt * pz * g;
    }
}

// ---- Esirkepov deposit --------------------------------------------------------
// Per dimension: old shape S0 at offsets 1..3 of a 5-point window starting two
// nodes below the old node, new shape S1 shifted by (new node - old node);
// A = (S0 + S1)/2 and D = S1 - S0.  The weight of the running sum is
// W(j,k) = A_j A_k + D_j D_k / 12, identical to the reference's
// S0 S0 + D S0/2 + S0 D/2 + D D/3 (Projector3D2Order.cpp:180-340).
struct Shape5 {
    double S0[5], S1[5], D[5];
};

__device__ __forceinline__ void shapes( double d_old, double xn, int ipo_global, Shape5 &s, int &ok )
{
    const int ip = round_half_away( xn );
    const int shift = ip - ipo_global;
    if( shift < -1 || shift > 1 ) ok = 0;
    const int sh = shift < -1 ? -1 : ( shift > 1 ? 1 : shift );
    double c0, c1, c2;
#pragma unroll
    for( int i = 0; i < 5; i++ ) { s.S0[i] = 0.0; s.S1[i] = 0.0; }
    bspline2( d_old, c0, c1, c2 );
    s.S0[1] = c0; s.S0[2] = c1; s.S0[3] = c2;
    bspline2( xn - ( double )ip, c0, c1, c2 );
    s.S1[sh + 1] = c0; s.S1[sh + 2] = c1; s.S1[sh + 3] = c2;
#pragma unroll
    for( int i = 0; i < 5; i++ ) s.D[i] = s.S1[i] - s.S0[i];
}

__device__ __forceinline__ void add_if( double *a, double v )
{
    if( v != 0.0 ) atomicAdd( a, v );
}

template <int DIM, int MODE>
__global__ void k_project( Dims d, double dt, double inv_vol, double3 dx_ov_dt, int64_t n,
                           const double *__restrict__ pos, const double *__restrict__ mom,
                           const double *__restrict__ weight, const short *__restrict__ charge,
                           const double *__restrict__ invgf, const int *__restrict__ iold,
                           const double *__restrict__ delta, double *Jx, double *Jy, double *Jz, double *rho,
                           int *status )
{
    const int64_t p = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x;
    if( p >= n ) return;
    const double cw = inv_vol * ( double )charge[p] * weight[p];
    const int nyp = d.nyp, nzp = d.nzp;
    if( MODE == 2 ) {
        double S[3][5];
        int base[3];
#pragma unroll
        for( int k = 0; k < DIM; k++ ) {
            const double xn = pos[k * n + p] * d.dxi[k];
            const int ip = round_half_away( xn );
            double c0, c1, c2;
            bspline2( xn - ( double )ip, c0, c1, c2 );
            S[k][0] = 0.0; S[k][1] = c0; S[k][2] = c1; S[k][3] = c2; S[k][4] = 0.0;
            base[k] = ip - d.db[k] - 2;
            const int np = k == 0 ? d.nxp : ( k == 1 ? d.nyp : d.nzp );
            if( base[k] < 0 || base[k] + 4 > np - 1 ) {
                atomicExch( &g_bounds_flag, 1 );
                return;
            }
        }
        if( DIM == 3 ) {
            for( int i = 1; i < 4; i++ )
                for( int j = 1; j < 4; j++ )
                    for( int k = 1; k < 4; k++ )
                        atomicAdd( &rho[lin( base[0] + i, base[1] + j, base[2] + k, nyp, nzp )], cw * S[0][i] * S[1][j] * S[2][k] );
        } else {
            for( int i = 1; i < 4; i++ )
                for( int j = 1; j < 4; j++ )
                    atomicAdd( &rho[( int64_t )( base[0] + i ) * nyp + base[1] + j], cw * S[0][i] * S[1][j] );
        }
        return;
    }
    Shape5 s[DIM];
    int base[3], ok = 1;
#pragma unroll
    for( int k = 0; k < DIM; k++ ) {
        const int ipo = iold[k * n + p];
        shapes( delta[k * n + p], pos[k * n + p] * d.dxi[k], ipo + d.db[k], s[k], ok );
        base[k] = ipo - 2;
        const int np = k == 0 ? d.nxp : ( k == 1 ? d.nyp : d.nzp );
        if( base[k] < 0 || base[k] + 4 > np - 1 ) {
            atomicExch( &g_bounds_flag, 1 );
            return;
        }
    }
    if( !ok ) atomicCAS( status, 0, SG_ERR_BOUNDS );
    if( DIM == 3 ) {
        const double cr[3] = { cw * dx_ov_dt.x, cw * dx_ov_dt.y, cw * dx_ov_dt.z };
        const int nyd = nyp + 1, nzd = nzp + 1;
        const double third = 1.0 / 3.0;
        for( int j = 0; j < 5; j++ )
            for( int k = 0; k < 5; k++ ) {
                const double w = s[1].S0[j] * s[2].S0[k] + 0.5 * s[1].D[j] * s[2].S0[k] + 0.5 * s[2].D[k] * s[1].S0[j] + third * s[1].D[j] * s[2].D[k];
                if( w == 0.0 ) continue;
                double acc = 0.0;
                for( int i = 1; i < 5; i++ ) {
                    acc -= cr[0] * s[0].D[i - 1] * w;
                    add_if( &Jx[lin( base[0] + i, base[1] + j, base[2] + k, nyp, nzp )], acc );
                }
            }
        for( int i = 0; i < 5; i++ )
            for( int k = 0; k < 5; k++ ) {
                const double w = s[2].S0[k] * s[0].S0[i] + 0.5 * s[2].D[k] * s[0].S0[i] + 0.5 * s[0].D[i] * s[2].S0[k] + third * s[2].D[k] * s[0].D[i];
                if( w == 0.0 ) continue;
                double acc = 0.0;
                for( int j = 1; j < 5; j++ ) {
                    acc -= cr[1] * s[1].D[j - 1] * w;
                    add_if( &Jy[lin( base[0] + i, base[1] + j, base[2] + k, nyd, nzp )], acc );
                }
            }
        for( int i = 0; i < 5; i++ )
            for( int j = 0; j < 5; j++ ) {
                const double w = s[0].S0[i] * s[1].S0[j] + 0.5 * s[0].D[i] * s[1].S0[j] + 0.5 * s[1].D[j] * s[0].S0[i] + third * s[0].D[i] * s[1].D[j];
                if( w == 0.0 ) continue;
                double acc = 0.0;
                for( int k = 1; k < 5; k++ ) {
                    acc -= cr[2] * s[2].D[k - 1] * w;
                    add_if( &Jz[lin( base[0] + i, base[1] + j, base[2] + k, nyp, nzd )], acc );
                }
            }
        if( MODE == 1 ) {
            for( int i = 0; i < 5; i++ )
                for( int j = 0; j < 5; j++ )
                    for( int k = 0; k < 5; k++ )
                        add_if( &rho[lin( base[0] + i, base[1] + j, base[2] + k, nyp, nzp )], cw * s[0].S1[i] * s[1].S1[j] * s[2].S1[k] );
        }
    } else {
        const double crx = cw * dx_ov_dt.x, cry = cw * dx_ov_dt.y;
        const double crz = cw * ( 1.0 / 3.0 ) * mom[2 * n + p] * invgf[p];
        const int nyd = nyp + 1;
        for( int j = 0; j < 5; j++ ) {
            const double w = s[1].S0[j] + 0.5 * s[1].D[j];
            double acc = 0.0;
            for( int i = 1; i < 5; i++ ) {
                acc -= crx * s[0].D[i - 1] * w;
                add_if( &Jx[( int64_t )( base[0] + i ) * nyp + base[1] + j], acc );
            }
        }
        for( int i = 0; i < 5; i++ ) {
            const double w = s[0].S0[i] + 0.5 * s[0].D[i];
            double acc = 0.0;
            for( int j = 1; j < 5; j++ ) {
                acc -= cry * s[1].D[j - 1] * w;
                add_if( &Jy[( int64_t )( base[0] + i ) * nyd + base[1] + j], acc );
            }
        }
        for( int i = 0; i < 5; i++ )
            for( int j = 0; j < 5; j++ ) {
                add_if( &Jz[( int64_t )( base[0] + i ) * nyp + base[1] + j],
                        crz * ( s[1].S0[j] * ( 0.5 * s[0].S1[i] + s[0].S0[i] ) + s[1].S1[j] * ( 0.5 * s[0].S0[i] + s[0].S1[i] ) ) );
                if( MODE == 1 ) add_if( &rho[( int64_t )( base[0] + i ) * nyp + base[1] + j], cw * s[0].S1[i] * s[1].S1[j] );
            }
    }
}

// ---- Yee ----------------------------------------------------------------------
// One thread per point of the component's extent (x slowest).  The 2D forms
// use nz = 1 and skip the z terms.
template <int DIM>
__global__ void k_ampere( int comp, int nx, int ny, int nz, int nyp, int nzp, double dt, double dtdx, double dtdy,
                          double dtdz, double *__restrict__ Ex, double *__restrict__ Ey, double *__restrict__ Ez,
                          const double *__restrict__ Bx, const double *__restrict__ By,
                          const double *__restrict__ Bz, const double *__restrict__ Jx,
                          const double *__restrict__ Jy, const double *__restrict__ Jz )
{
    const int64_t t = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x;
    if( t >= ( int64_t )nx * ny * nz ) return;
    const int k = ( int )( t % nz ), j = ( int )( ( t / nz ) % ny ), i = ( int )( t / ( ( int64_t )nz * ny ) );
    const int nyd = nyp + 1, nzd = DIM == 3 ? nzp + 1 : 1;
    if( DIM == 3 ) {
        if( comp == 0 )
            Ex[t] += -dt * Jx[t] + dtdy * ( Bz[lin( i, j + 1, k, nyd, nzp )] - Bz[lin( i, j, k, nyd, nzp )] )
                     - dtdz * ( By[lin( i, j, k + 1, nyp, nzd )] - By[lin( i, j, k, nyp, nzd )] );
        else if( comp == 1 )
            Ey[t] += -dt * Jy[t] - dtdx * ( Bz[lin( i + 1, j, k, nyd, nzp )] - Bz[lin( i, j, k, nyd, nzp )] )
                     + dtdz * ( Bx[lin( i, j, k + 1, nyd, nzd )] - Bx[lin( i, j, k, nyd, nzd )] );
        else
            Ez[t] += -dt * Jz[t] + dtdx * ( By[lin( i + 1, j, k, nyp, nzd )] - By[lin( i, j, k, nyp, nzd )] )
                     - dtdy * ( Bx[lin( i, j + 1, k, nyd, nzd )] - Bx[lin( i, j, k, nyd, nzd )] );
    } else {
        if( comp == 0 )
            Ex[t] += -dt * Jx[t] + dtdy * ( Bz[( int64_t )i * nyd + j + 1] - Bz[( int64_t )i * nyd + j] );
        else if( comp == 1 )
            Ey[t] += -dt * Jy[t] - dtdx * ( Bz[( int64_t )( i + 1 ) * nyd + j] - Bz[( int64_t )i * nyd + j] );
        else
            Ez[t] += -dt * Jz[t] + dtdx * ( By[( int64_t )( i + 1 ) * nyp + j] - By[( int64_t )i * nyp + j] )
                     - dtdy * ( Bx[( int64_t )i * nyd + j + 1] - Bx[( int64_t )i * nyd + j] );
    }
}

// Faraday on interior points: the thread grid covers the component's extent
// and the boundary layers of its dual dimensions are skipped.
template <int DIM>
__global__ void k_faraday( int comp, int nx, int ny, int nz, int nyp, int nzp, double dtdx, double dtdy, double dtdz,
                           const double *__restrict__ Ex, const double *__restrict__ Ey,
                           const double *__restrict__ Ez, double *__restrict__ Bx, double *__restrict__ By,
                           double *__restrict__ Bz )
{
    const int64_t t = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x;
    if( t >= ( int64_t )nx * ny * nz ) return;
    const int k = ( int )( t % nz ), j = ( int )( ( t / nz ) % ny ), i = ( int )( t / ( ( int64_t )nz * ny ) );
    const int nyd = nyp + 1, nzd = DIM == 3 ? nzp + 1 : 1;
    if( DIM == 3 ) {
        if( comp == 0 ) {
            if( j < 1 || j >= ny - 1 || k < 1 || k >= nz - 1 ) return;
            Bx[t] += -dtdy * ( Ez[lin( i, j, k, nyp, nzd )] - Ez[lin( i, j - 1, k, nyp, nzd )] )
                     + dtdz * ( Ey[lin( i, j, k, nyd, nzp )] - Ey[lin( i, j, k - 1, nyd, nzp )] );
        } else if( comp == 1 ) {
            if( i < 1 || i >= nx - 1 || k < 1 || k >= nz - 1 ) return;
            By[t] += -dtdz * ( Ex[lin( i, j, k, nyp, nzp )] - Ex[lin( i, j, k - 1, nyp, nzp )] )
                     + dtdx * ( Ez[lin( i, j, k, nyp, nzd )] - Ez[lin( i - 1, j, k, nyp, nzd )] );
        } else {
            if( i < 1 || i >= nx - 1 || j < 1 || j >= ny - 1 ) return;
            Bz[t] += -dtdx * ( Ey[lin( i, j, k, nyd, nzp )] - Ey[lin( i - 1, j, k, nyd, nzp )] )
                     + dtdy * ( Ex[lin( i, j, k, nyp, nzp )] - Ex[lin( i, j - 1, k, nyp, nzp )] );
        }
    } else {
        if( comp == 0 ) {
            if( j < 1 || j >= ny - 1 ) return;
            Bx[t] -= dtdy * ( Ez[( int64_t )i * nyp + j] - Ez[( int64_t )i * nyp + j - 1] );
        } else if( comp == 1 ) {
            if( i < 1 || i >= nx - 1 ) return;
            By[t] += dtdx * ( Ez[( int64_t )i * nyp + j] - Ez[( int64_t )( i - 1 ) * nyp + j] );
        } else {
            if( i < 1 || i >= nx - 1 || j < 1 || j >= ny - 1 ) return;
            Bz[t] += dtdy * ( Ex[( int64_t )i * nyp + j] - Ex[( int64_t )i * nyp + j - 1] )
                     - dtdx * ( Ey[( int64_t )i * nyd + j] - Ey[( int64_t )( i - 1 ) * nyd + j] );
        }
    }
}

__global__ void k_save_b( int64_t n, const double *__restrict__ B, double *__restrict__ Bm )
{
    const int64_t t = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x;
    if( t < n ) Bm[t] = B[t];
}

__global__ void k_center_b( int64_t n, const double *__restrict__ B, double *__restrict__ Bm )
{
    const int64_t t = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x;
    if( t < n ) Bm[t] = ( B[t] + Bm[t] ) * 0.5;
}

int check_geom( const sg_grid_geom *g )
{
    SG_REQUIRE( g != nullptr, "geometry is NULL" );
    SG_REQUIRE( g->ndim == 2 || g->ndim == 3, "ndim must be 2 or 3 (got %d)", g->ndim );
    for( int d = 0; d < g->ndim; d++ ) {
        SG_REQUIRE( g->n_prim[d] >= 6, "n_prim[%d] = %d is too small", d, g->n_prim[d] );
        SG_REQUIRE( g->cell_length[d] > 0.0, "cell_length[%d] must be positive", d );
    }
    return SG_OK;
}

// Extents of a component with staggering (sx, sy, sz).
void comp_extent( const sg_grid_geom *g, int sx, int sy, int sz, int &nx, int &ny, int &nz )
{
    nx = g->n_prim[0] + sx;
    ny = g->n_prim[1] + sy;
    nz = g->ndim == 3 ? g->n_prim[2] + sz : 1;
}

} // namespace

int set_error( int code, const char *fmt, ... )
{
    char buf[1024];
    va_list ap;
    va_start( ap, fmt );
    vsnprintf( buf, sizeof( buf ), fmt, ap );
    va_end( ap );
    g_last_error = buf;
    return code;
}

} // namespace sg

using namespace sg;

extern "C" {

const char *sg_last_error( void ) { return g_last_error.c_str(); }

int sg_version( void ) { return 10000; }

int sg_interpolate_fields( const sg_grid_geom *geom, const double *const *fields, int64_t npart, const double *pos,
                           double *Epart, double *Bpart, int *iold, double *deltaold, sg_stream_t stream )
{
    int st = check_geom( geom );
    if( st ) return st;
    SG_REQUIRE( npart >= 0, "npart < 0" );
    if( npart == 0 ) return SG_OK;
    SG_REQUIRE( fields && pos && Epart && Bpart && iold && deltaold, "NULL array" );
    Dims d = make_dims( geom );
    const int B = 128;
    if( geom->ndim == 3 )
        k_interpolate<3><<<grid_for( npart, B ), B, 0, as_stream( stream )>>>( d, fields[0], fields[1], fields[2], fields[3], fields[4], fields[5], npart, pos, Epart, Bpart, iold, deltaold );
    else
        k_interpolate<2><<<grid_for( npart, B ), B, 0, as_stream( stream )>>>( d, fields[0], fields[1], fields[2], fields[3], fields[4], fields[5], npart, pos, Epart, Bpart, iold, deltaold );
    SG_LAUNCH_CHECK( "k_interpolate" );
    return SG_OK;
}

int sg_push_particles( int kind, int ndim, double dt, double mass, int64_t npart, double *pos, double *mom,
                       const short *charge, const double *Epart, const double *Bpart, double *invgf,
                       sg_stream_t stream )
{
    SG_REQUIRE( kind >= 0 && kind <= 2, "pusher kind must be 0 (boris), 1 (vay) or 2 (higueracary)" );
    SG_REQUIRE( ndim >= 1 && ndim <= 3, "ndim must be 1..3" );
    SG_REQUIRE( npart >= 0, "npart < 0" );
    if( npart == 0 ) return SG_OK;
    SG_REQUIRE( pos && mom && charge && Epart && Bpart && invgf, "NULL array" );
    const double oom = mass > 0.0 ? 1.0 / mass : 0.0;
    const int B = 256;
    cudaStream_t s = as_stream( stream );
    if( kind == 0 ) k_push<0><<<grid_for( npart, B ), B, 0, s>>>( ndim, dt, oom, npart, pos, mom, charge, Epart, Bpart, invgf );
    else if( kind == 1 ) k_push<1><<<grid_for( npart, B ), B, 0, s>>>( ndim, dt, oom, npart, pos, mom, charge, Epart, Bpart, invgf );
    else k_push<2><<<grid_for( npart, B ), B, 0, s>>>( ndim, dt, oom, npart, pos, mom, charge, Epart, Bpart, invgf );
    SG_LAUNCH_CHECK( "k_push" );
    return SG_OK;
}

int sg_project_currents( int mode, const sg_grid_geom *geom, double dt, int64_t npart, const double *pos,
                         const double *mom, const double *weight, const short *charge, const double *invgf,
                         const int *iold, const double *deltaold, double *const *J, sg_stream_t stream )
{
    int st = check_geom( geom );
    if( st ) return st;
    SG_REQUIRE( mode >= 0 && mode <= 2, "mode must be 0, 1 or 2" );
    SG_REQUIRE( npart >= 0, "npart < 0" );
    if( npart == 0 ) return SG_OK;
    SG_REQUIRE( J && pos && weight && charge, "NULL array" );
    if( mode != 2 ) SG_REQUIRE( J[0] && J[1] && J[2] && iold && deltaold, "currents need Jx, Jy, Jz, iold, deltaold" );
    if( mode != 0 ) SG_REQUIRE( J[3] != nullptr, "rho is NULL" );
    if( mode != 2 && geom->ndim == 2 ) SG_REQUIRE( mom && invgf, "2D currents need momenta and invgf" );
    Dims d = make_dims( geom );
    double vol = 1.0;
    for( int k = 0; k < geom->ndim; k++ ) vol *= geom->cell_length[k];
    double3 dxdt = make_double3( geom->cell_length[0] / dt, geom->cell_length[1] / dt,
                                 geom->ndim == 3 ? geom->cell_length[2] / dt : 0.0 );
    int *status = nullptr;
    cudaStream_t s = as_stream( stream );
    SG_CUDA_TRY( cudaMallocAsync( &status, sizeof( int ), s ) );
    SG_CUDA_TRY( cudaMemsetAsync( status, 0, sizeof( int ), s ) );
    const int B = 128;
    const unsigned g = grid_for( npart, B );
#define SG_PROJ( D, M ) k_project<D, M><<<g, B, 0, s>>>( d, dt, 1.0 / vol, dxdt, npart, pos, mom, weight, charge, invgf, iold, deltaold, J[0], J[1], J[2], J[3], status )
    if( geom->ndim == 3 ) {
        if( mode == 0 ) SG_PROJ( 3, 0 ); else if( mode == 1 ) SG_PROJ( 3, 1 ); else SG_PROJ( 3, 2 );
    } else {
        if( mode == 0 ) SG_PROJ( 2, 0 ); else if( mode == 1 ) SG_PROJ( 2, 1 ); else SG_PROJ( 2, 2 );
    }
#undef SG_PROJ
    SG_LAUNCH_CHECK( "k_project" );
    int h_status = 0;
    SG_CUDA_TRY( cudaMemcpyAsync( &h_status, status, sizeof( int ), cudaMemcpyDeviceToHost, s ) );
    SG_CUDA_TRY( cudaFreeAsync( status, s ) );
    SG_CUDA_TRY( cudaStreamSynchronize( s ) );
    int h_bounds = 0, zero = 0;
    SG_CUDA_TRY( cudaMemcpyFromSymbol( &h_bounds, g_bounds_flag, sizeof( int ) ) );
    if( h_bounds ) SG_CUDA_TRY( cudaMemcpyToSymbol( g_bounds_flag, &zero, sizeof( int ) ) );
    if( h_status ) return set_error( h_status, "a particle moved more than one cell during the step (Esirkepov stencil exceeded)" );
    if( h_bounds ) return set_error( SG_ERR_BOUNDS, "a particle's stencil left the patch arrays (gather or deposit); its contribution was skipped" );
    return SG_OK;
}

int sg_maxwell_ampere( const sg_grid_geom *geom, double dt, double *const *F, sg_stream_t stream )
{
    int st = check_geom( geom );
    if( st ) return st;
    SG_REQUIRE( F != nullptr, "NULL field list" );
    for( int c = 0; c < 9; c++ ) SG_REQUIRE( F[c] != nullptr, "field %d is NULL", c );
    const double dtdx = dt / geom->cell_length[0], dtdy = dt / geom->cell_length[1];
    const double dtdz = geom->ndim == 3 ? dt / geom->cell_length[2] : 0.0;
    const int nyp = geom->n_prim[1], nzp = geom->ndim == 3 ? geom->n_prim[2] : 1;
    static const int stag[3][3] = { { 1, 0, 0 }, { 0, 1, 0 }, { 0, 0, 1 } };
    cudaStream_t s = as_stream( stream );
    for( int c = 0; c < 3; c++ ) {
        int nx, ny, nz;
        comp_extent( geom, stag[c][0], stag[c][1], stag[c][2], nx, ny, nz );
        const int64_t n = ( int64_t )nx * ny * nz;
        if( geom->ndim == 3 )
            k_ampere<3><<<grid_for( n, 256 ), 256, 0, s>>>( c, nx, ny, nz, nyp, nzp, dt, dtdx, dtdy, dtdz, F[0], F[1], F[2], F[3], F[4], F[5], F[6], F[7], F[8] );
        else
            k_ampere<2><<<grid_for( n, 256 ), 256, 0, s>>>( c, nx, ny, nz, nyp, nzp, dt, dtdx, dtdy, dtdz, F[0], F[1], F[2], F[3], F[4], F[5], F[6], F[7], F[8] );
        SG_LAUNCH_CHECK( "k_ampere" );
    }
    return SG_OK;
}

int sg_maxwell_faraday( const sg_grid_geom *geom, double dt, double *const *F, sg_stream_t stream )
{
    int st = check_geom( geom );
    if( st ) return st;
    SG_REQUIRE( F != nullptr, "NULL field list" );
    for( int c = 0; c < 6; c++ ) SG_REQUIRE( F[c] != nullptr, "field %d is NULL", c );
    const double dtdx = dt / geom->cell_length[0], dtdy = dt / geom->cell_length[1];
    const double dtdz = geom->ndim == 3 ? dt / geom->cell_length[2] : 0.0;
    const int nyp = geom->n_prim[1], nzp = geom->ndim == 3 ? geom->n_prim[2] : 1;
    static const int stag[3][3] = { { 0, 1, 1 }, { 1, 0, 1 }, { 1, 1, 0 } };
    cudaStream_t s = as_stream( stream );
    for( int c = 0; c < 3; c++ ) {
        int nx, ny, nz;
        comp_extent( geom, stag[c][0], stag[c][1], stag[c][2], nx, ny, nz );
        const int64_t n = ( int64_t )nx * ny * nz;
        if( geom->ndim == 3 )
            k_faraday<3><<<grid_for( n, 256 ), 256, 0, s>>>( c, nx, ny, nz, nyp, nzp, dtdx, dtdy, dtdz, F[0], F[1], F[2], F[3], F[4], F[5] );
        else
            k_faraday<2><<<grid_for( n, 256 ), 256, 0, s>>>( c, nx, ny, nz, nyp, nzp, dtdx, dtdy, dtdz, F[0], F[1], F[2], F[3], F[4], F[5] );
        SG_LAUNCH_CHECK( "k_faraday" );
    }
    return SG_OK;
}

static int b_op( const sg_grid_geom *geom, double *const *B, double *const *Bm, bool center, sg_stream_t stream )
{
    int st = check_geom( geom );
    if( st ) return st;
    SG_REQUIRE( B && Bm, "NULL field list" );
    static const int stag[3][3] = { { 0, 1, 1 }, { 1, 0, 1 }, { 1, 1, 0 } };
    cudaStream_t s = as_stream( stream );
    for( int c = 0; c < 3; c++ ) {
        SG_REQUIRE( B[c] && Bm[c], "component %d is NULL", c );
        int nx, ny, nz;
        comp_extent( geom, stag[c][0], stag[c][1], stag[c][2], nx, ny, nz );
        const int64_t n = ( int64_t )nx * ny * nz;
        if( center ) k_center_b<<<grid_for( n, 256 ), 256, 0, s>>>( n, B[c], Bm[c] );
        else k_save_b<<<grid_for( n, 256 ), 256, 0, s>>>( n, B[c], Bm[c] );
        SG_LAUNCH_CHECK( "k_center_b" );
    }
    return SG_OK;
}

int sg_save_magnetic_fields( const sg_grid_geom *geom, double *const *B, double *const *Bm, sg_stream_t stream )
{
    return b_op( geom, B, Bm, false, stream );
}

int sg_center_magnetic_fields( const sg_grid_geom *geom, double *const *B, double *const *Bm, sg_stream_t stream )
{
    return b_op( geom, B, Bm, true, stream );
}

} // extern "C"
