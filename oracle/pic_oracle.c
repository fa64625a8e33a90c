/* pic_oracle.c -- CPU restatement of the reference's PIC-step operators.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.  The product
 * (smilei_gb300/, libsmileigb300.so) never links or calls it.
 *
 * Everything is plain FP64 C, one function per reference operator, on the
 * reference's own data layout:
 *   - fields: x-major, last dimension fastest; a primal dimension has
 *     n_cells + 1 + 2*oversize points, a dual one has one more
 *     (ElectroMagn3D.cpp:115-123, Params.cpp:1202-1207);
 *   - Yee staggering Ex(d,p,p) Ey(p,d,p) Ez(p,p,d) Bx(p,d,d) By(d,p,d) Bz(d,d,p),
 *     J like E, rho primal; in 2D the third index is dropped (Ez, Jz (p,p); Bz (d,d));
 *   - particles: SoA, absolute positions pos[d*n + i], momenta mom[d*n + i];
 *   - interpolator scratch Epart/Bpart[3n], iold/delta[ndim*n] (SmileiMPI.h:213-221).
 * The results are pinned against the reference's compiled operators by the
 * golden fixtures in tests/golden (made by tests/golden/make_golden.py from
 * oracle/_ref/libsmilei_ref_ops.so).  Build with -ffp-contract=off so x86 and
 * Arm hosts give the same bits.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_ONE_THIRD ( 1.0 / 3.0 )

/* Index of (i,j,k) in an array of extents (.., ny, nz); 2D arrays pass nz = 1, k = 0. */
static inline int64_t lin3( int i, int j, int k, int ny, int nz )
{
    return ( ( int64_t )i * ny + j ) * nz + k;
}

/* Quadratic B-spline weights at offsets -1, 0, +1 for an in-cell offset d
 * (Interpolator3D2Order.h:109-125). */
static inline void bspline2( double d, double *c )
{
    const double d2 = d * d;
    c[0] = 0.5 * ( d2 - d + 0.25 );
    c[1] = 0.75 - d2;
    c[2] = 0.5 * ( d2 + d + 0.25 );
}

/* ------------------------------------------------------------------------- */
/* Interpolator{2D,3D}2Order::fieldsWrapper                                   */
/* Interpolator3D2Order.cpp:163-285 (coeffs .h:95-158, compute .h:54-76);     */
/* Interpolator2D2Order.cpp:158-290 (coeffs .h:92-150).                       */
/* fields = {Ex, Ey, Ez, Bx_m, By_m, Bz_m}; n_prim = primal extents with       */
/* ghosts; domain_begin = patch start minus oversize (Interpolator3D.cpp:14). */
/* ------------------------------------------------------------------------- */
static double gather3( const double *f, const double *cx, const double *cy, const double *cz, int i, int j, int k,
                       int ny, int nz )
{
    double r = 0.0;
    for( int a = -1; a < 2; a++ )
        for( int b = -1; b < 2; b++ )
            for( int c = -1; c < 2; c++ ) r += cx[a + 1] * cy[b + 1] * cz[c + 1] * f[lin3( i + a, j + b, k + c, ny, nz )];
    return r;
}

static double gather2( const double *f, const double *cx, const double *cy, int i, int j, int ny )
{
    double r = 0.0;
    for( int a = -1; a < 2; a++ )
        for( int b = -1; b < 2; b++ ) r += cx[a + 1] * cy[b + 1] * f[( int64_t )( i + a ) * ny + ( j + b )];
    return r;
}

int or_interpolate( int ndim, const int *n_prim, const int *domain_begin, const double *dx_inv,
                    const double *const *fields, int64_t npart, const double *pos, double *Epart, double *Bpart,
                    int *iold, double *delta )
{
    const double *Ex = fields[0], *Ey = fields[1], *Ez = fields[2];
    const double *Bx = fields[3], *By = fields[4], *Bz = fields[5];
    const int nxp = n_prim[0], nyp = n_prim[1], nzp = ndim == 3 ? n_prim[2] : 1;
    const int nyd = nyp + 1, nzd = nzp + 1;
    ( void )nxp;
#pragma omp parallel for schedule( static )
    for( int64_t p = 0; p < npart; p++ ) {
        int ip[3], id[3];
        double cp[3][3], cd[3][3], dp[3];
        for( int d = 0; d < ndim; d++ ) {
            const double xn = pos[d * npart + p] * dx_inv[d];
            ip[d] = ( int )round( xn );
            dp[d] = xn - ( double )ip[d];
            bspline2( dp[d], cp[d] );
            id[d] = ( int )round( xn + 0.5 );
            bspline2( xn - ( double )id[d] + 0.5, cd[d] );
            ip[d] -= domain_begin[d];
            id[d] -= domain_begin[d];
        }
        if( ndim == 3 ) {
            Epart[0 * npart + p] = gather3( Ex, cd[0], cp[1], cp[2], id[0], ip[1], ip[2], nyp, nzp );
            Epart[1 * npart + p] = gather3( Ey, cp[0], cd[1], cp[2], ip[0], id[1], ip[2], nyd, nzp );
            Epart[2 * npart + p] = gather3( Ez, cp[0], cp[1], cd[2], ip[0], ip[1], id[2], nyp, nzd );
            Bpart[0 * npart + p] = gather3( Bx, cp[0], cd[1], cd[2], ip[0], id[1], id[2], nyd, nzd );
            Bpart[1 * npart + p] = gather3( By, cd[0], cp[1], cd[2], id[0], ip[1], id[2], nyp, nzd );
            Bpart[2 * npart + p] = gather3( Bz, cd[0], cd[1], cp[2], id[0], id[1], ip[2], nyd, nzp );
        } else {
            Epart[0 * npart + p] = gather2( Ex, cd[0], cp[1], id[0], ip[1], nyp );
            Epart[1 * npart + p] = gather2( Ey, cp[0], cd[1], ip[0], id[1], nyd );
            Epart[2 * npart + p] = gather2( Ez, cp[0], cp[1], ip[0], ip[1], nyp );
            Bpart[0 * npart + p] = gather2( Bx, cp[0], cd[1], ip[0], id[1], nyd );
            Bpart[1 * npart + p] = gather2( By, cd[0], cp[1], id[0], ip[1], nyp );
            Bpart[2 * npart + p] = gather2( Bz, cd[0], cd[1], id[0], id[1], nyd );
        }
        for( int d = 0; d < ndim; d++ ) {
            iold[d * npart + p] = ip[d];
            delta[d * npart + p] = dp[d];
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Pushers. kind 0: Boris (PusherBoris.cpp:82-127); 1: Vay (PusherVay.cpp:92-  */
/* 173); 2: Higuera-Cary (PusherHigueraCary.cpp:93-167).  Constants from       */
/* Pusher.cpp:5-29: one_over_mass = 1/m, dts2 = dt/2.                           */
/* ------------------------------------------------------------------------- */
int or_push( int kind, int ndim, double dt, double mass, int64_t npart, double *pos, double *mom, const short *charge,
             const double *Epart, const double *Bpart, double *invgf )
{
    const double one_over_mass = mass > 0.0 ? 1.0 / mass : 0.0;
    const double dts2 = dt / 2.0;
#pragma omp parallel for schedule( static )
    for( int64_t p = 0; p < npart; p++ ) {
        const double qm = ( double )charge[p] * one_over_mass * dts2;
        const double Ex = Epart[p], Ey = Epart[npart + p], Ez = Epart[2 * npart + p];
        const double Bx = Bpart[p], By = Bpart[npart + p], Bz = Bpart[2 * npart + p];
        double px = mom[p], py = mom[npart + p], pz = mom[2 * npart + p];
        double g_inv;
        if( kind == 0 ) {
            double pxsm = qm * Ex, pysm = qm * Ey, pzsm = qm * Ez;
            const double umx = px + pxsm, umy = py + pysm, umz = pz + pzsm;
            const double lg = qm / sqrt( 1.0 + umx * umx + umy * umy + umz * umz );
            const double Tx = lg * Bx, Ty = lg * By, Tz = lg * Bz;
            const double inv_det = 1.0 / ( 1.0 + Tx * Tx + Ty * Ty + Tz * Tz );
            pxsm += ( ( 1.0 + Tx * Tx - Ty * Ty - Tz * Tz ) * umx + 2.0 * ( Tx * Ty + Tz ) * umy + 2.0 * ( Tz * Tx - Ty ) * umz ) * inv_det;
            pysm += ( 2.0 * ( Tx * Ty - Tz ) * umx + ( 1.0 - Tx * Tx + Ty * Ty - Tz * Tz ) * umy + 2.0 * ( Ty * Tz + Tx ) * umz ) * inv_det;
            pzsm += ( 2.0 * ( Tz * Tx + Ty ) * umx + 2.0 * ( Ty * Tz - Tx ) * umy + ( 1.0 - Tx * Tx - Ty * Ty + Tz * Tz ) * umz ) * inv_det;
            g_inv = 1.0 / sqrt( 1.0 + pxsm * pxsm + pysm * pysm + pzsm * pzsm );
            px = pxsm; py = pysm; pz = pzsm;
        } else if( kind == 1 ) {
            const double g0 = 1.0 / sqrt( 1.0 + px * px + py * py + pz * pz );
            double upx = px + 2.0 * qm * Ex, upy = py + 2.0 * qm * Ey, upz = pz + 2.0 * qm * Ez;
            double Tx = qm * Bx, Ty = qm * By, Tz = qm * Bz;
            upx += g0 * ( py * Tz - pz * Ty );
            upy += g0 * ( pz * Tx - px * Tz );
            upz += g0 * ( px * Ty - py * Tx );
            double alpha = 1.0 + upx * upx + upy * upy + upz * upz;
            const double T2 = Tx * Tx + Ty * Ty + Tz * Tz;
            double s = alpha - T2;
            double us2 = upx * Tx + upy * Ty + upz * Tz;
            us2 = us2 * us2;
            alpha = 1.0 / sqrt( 0.5 * ( s + sqrt( s * s + 4.0 * ( T2 + us2 ) ) ) );
            Tx *= alpha; Ty *= alpha; Tz *= alpha;
            s = 1.0 / ( 1.0 + Tx * Tx + Ty * Ty + Tz * Tz );
            alpha = upx * Tx + upy * Ty + upz * Tz;
            px = s * ( upx + alpha * Tx + Tz * upy - Ty * upz );
            py = s * ( upy + alpha * Ty + Tx * upz - Tz * upx );
            pz = s * ( upz + alpha * Tz + Ty * upx - Tx * upy );
            g_inv = 1.0 / sqrt( 1.0 + px * px + py * py + pz * pz );
        } else {
            double pxsm = qm * Ex, pysm = qm * Ey, pzsm = qm * Ez;
            const double umx = px + pxsm, umy = py + pysm, umz = pz + pzsm;
            const double gfm2 = 1.0 + umx * umx + umy * umy + umz * umz;
            double Tx = qm * Bx, Ty = qm * By, Tz = qm * Bz;
            const double beta2 = Tx * Tx + Ty * Ty + Tz * Tz;
            const double Tum = Tx * umx + Ty * umy + Tz * umz;
            const double lg = 1.0 / sqrt( 0.5 * ( gfm2 - beta2 + sqrt( ( gfm2 - beta2 ) * ( gfm2 - beta2 ) + 4.0 * ( beta2 + Tum * Tum ) ) ) );
            Tx *= lg; Ty *= lg; Tz *= lg;
            const double Tx2 = Tx * Tx, Ty2 = Ty * Ty, Tz2 = Tz * Tz;
            const double TxTy = Tx * Ty, TyTz = Ty * Tz, TzTx = Tz * Tx;
            const double inv_det = 1.0 / ( 1.0 + Tx2 + Ty2 + Tz2 );
            const double upx = ( ( 1.0 + Tx2 - Ty2 - Tz2 ) * umx + 2.0 * ( TxTy + Tz ) * umy + 2.0 * ( TzTx - Ty ) * umz ) * inv_det;
            const double upy = ( 2.0 * ( TxTy - Tz ) * umx + ( 1.0 - Tx2 + Ty2 - Tz2 ) * umy + 2.0 * ( TyTz + Tx ) * umz ) * inv_det;
            const double upz = ( 2.0 * ( TzTx + Ty ) * umx + 2.0 * ( TyTz - Tx ) * umy + ( 1.0 - Tx2 - Ty2 + Tz2 ) * umz ) * inv_det;
            pxsm += upx; pysm += upy; pzsm += upz;
            g_inv = 1.0 / sqrt( 1.0 + pxsm * pxsm + pysm * pysm + pzsm * pzsm );
            px = pxsm; py = pysm; pz = pzsm;
        }
        invgf[p] = g_inv;
        mom[p] = px;
        mom[npart + p] = py;
        mom[2 * npart + p] = pz;
        if( kind == 0 ) {
            /* Boris folds dt into the inverse gamma first (PusherBoris.cpp:117). */
            const double vdt = g_inv * dt;
            pos[p] += px * vdt;
            if( ndim > 1 ) pos[npart + p] += py * vdt;
            if( ndim > 2 ) pos[2 * npart + p] += pz * vdt;
        } else {
            pos[p] += dt * px * g_inv;
            if( ndim > 1 ) pos[npart + p] += dt * py * g_inv;
            if( ndim > 2 ) pos[2 * npart + p] += dt * pz * g_inv;
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Esirkepov projection.                                                       */
/* 3D: Projector3D2Order::currents (Projector3D2Order.cpp:55-343),             */
/*     currentsAndDensity (:349-521), basic (:526-618).                        */
/* 2D: Projector2D2Order::currents (Projector2D2Order.cpp:49-186) and           */
/*     currentsAndDensity (:190-...).                                          */
/* charge_weight = q*w/V_cell (Projector.cpp:7); crx = cw*dx/dt;               */
/* 2D crz = cw*(1/3)*pz*invgf (Projector2D2Order.cpp:62).                       */
/* J = {Jx, Jy, Jz, rho}.  mode 0: J only; 1: J and rho; 2: rho only (basic).  */
/* Sequential over particles (the reference's CPU order).                      */
/* ------------------------------------------------------------------------- */
static void old_new_shapes( double d_old, double xn, int ipo_global, int *shift_out, double *S0, double *S1 )
{
    const int ip = ( int )round( xn );
    const int shift = ip - ipo_global;
    const double dn = xn - ( double )ip;
    double c[3];
    for( int i = 0; i < 5; i++ ) { S0[i] = 0.0; S1[i] = 0.0; }
    bspline2( d_old, c );
    S0[1] = c[0]; S0[2] = c[1]; S0[3] = c[2];
    bspline2( dn, c );
    S1[shift + 1] = c[0]; S1[shift + 2] = c[1]; S1[shift + 3] = c[2];
    *shift_out = shift;
}

static void project_range( int mode, int ndim, const int *n_prim, const int *domain_begin, const double *cell_length,
                           double dt, int64_t npart, const double *pos, const double *mom, const double *weight,
                           const short *charge, const double *invgf, const int *iold, const double *delta,
                           double *const *J, int64_t p_begin, int64_t p_end )
{
    double inv_vol = 1.0, dx_inv[3], dx_ov_dt[3];
    for( int d = 0; d < ndim; d++ ) {
        inv_vol *= cell_length[d];
        dx_inv[d] = 1.0 / cell_length[d];
        dx_ov_dt[d] = cell_length[d] / dt;
    }
    inv_vol = 1.0 / inv_vol;
    double *Jx = J[0], *Jy = J[1], *Jz = J[2], *rho = J[3];
    const int nxp = n_prim[0], nyp = n_prim[1], nzp = ndim == 3 ? n_prim[2] : 1;
    ( void )nxp;
    for( int64_t p = p_begin; p < p_end; p++ ) {
        const double cw = inv_vol * ( double )charge[p] * weight[p];
        if( mode == 2 ) {
            /* basic(): rho from the current position only. */
            double S[3][5];
            int base[3];
            for( int d = 0; d < ndim; d++ ) {
                const double xn = pos[d * npart + p] * dx_inv[d];
                const int ip = ( int )round( xn );
                double c[3];
                bspline2( xn - ( double )ip, c );
                S[d][0] = 0.0; S[d][1] = c[0]; S[d][2] = c[1]; S[d][3] = c[2]; S[d][4] = 0.0;
                base[d] = ip - domain_begin[d] - 2;
            }
            if( ndim == 3 ) {
                for( int i = 0; i < 5; i++ )
                    for( int j = 0; j < 5; j++ )
                        for( int k = 0; k < 5; k++ )
                            rho[lin3( base[0] + i, base[1] + j, base[2] + k, nyp, nzp )] += cw * S[0][i] * S[1][j] * S[2][k];
            } else {
                for( int i = 0; i < 5; i++ )
                    for( int j = 0; j < 5; j++ ) rho[( int64_t )( base[0] + i ) * nyp + base[1] + j] += cw * S[0][i] * S[1][j];
            }
            continue;
        }
        double S0[3][5], S1[3][5], DS[3][5];
        int base[3], shift;
        for( int d = 0; d < ndim; d++ ) {
            const int ipo = iold[d * npart + p];
            old_new_shapes( delta[d * npart + p], pos[d * npart + p] * dx_inv[d], ipo + domain_begin[d], &shift, S0[d], S1[d] );
            for( int i = 0; i < 5; i++ ) DS[d][i] = S1[d][i] - S0[d][i];
            base[d] = ipo - 2;
        }
        if( ndim == 3 ) {
            const double cr[3] = { cw * dx_ov_dt[0], cw * dx_ov_dt[1], cw * dx_ov_dt[2] };
            const int nyd = nyp + 1, nzd = nzp + 1;
            /* Jx(d,p,p): running sum over x of Wx = DSx*(Sy0 Sz0 + DSy Sz0/2 + Sy0 DSz/2 + DSy DSz/3). */
            for( int j = 0; j < 5; j++ )
                for( int k = 0; k < 5; k++ ) {
                    const double w = S0[1][j] * S0[2][k] + 0.5 * DS[1][j] * S0[2][k] + 0.5 * DS[2][k] * S0[1][j] + OR_ONE_THIRD * DS[1][j] * DS[2][k];
                    double acc = 0.0;
                    for( int i = 1; i < 5; i++ ) {
                        acc -= cr[0] * DS[0][i - 1] * w;
                        Jx[lin3( base[0] + i, base[1] + j, base[2] + k, nyp, nzp )] += acc;
                    }
                }
            for( int i = 0; i < 5; i++ )
                for( int k = 0; k < 5; k++ ) {
                    const double w = S0[2][k] * S0[0][i] + 0.5 * DS[2][k] * S0[0][i] + 0.5 * DS[0][i] * S0[2][k] + OR_ONE_THIRD * DS[2][k] * DS[0][i];
                    double acc = 0.0;
                    for( int j = 1; j < 5; j++ ) {
                        acc -= cr[1] * DS[1][j - 1] * w;
                        Jy[lin3( base[0] + i, base[1] + j, base[2] + k, nyd, nzp )] += acc;
                    }
                }
            for( int i = 0; i < 5; i++ )
                for( int j = 0; j < 5; j++ ) {
                    const double w = S0[0][i] * S0[1][j] + 0.5 * DS[0][i] * S0[1][j] + 0.5 * DS[1][j] * S0[0][i] + OR_ONE_THIRD * DS[0][i] * DS[1][j];
                    double acc = 0.0;
                    for( int k = 1; k < 5; k++ ) {
                        acc -= cr[2] * DS[2][k - 1] * w;
                        Jz[lin3( base[0] + i, base[1] + j, base[2] + k, nyp, nzd )] += acc;
                    }
                }
            if( mode == 1 ) {
                for( int i = 0; i < 5; i++ )
                    for( int j = 0; j < 5; j++ )
                        for( int k = 0; k < 5; k++ )
                            rho[lin3( base[0] + i, base[1] + j, base[2] + k, nyp, nzp )] += cw * S1[0][i] * S1[1][j] * S1[2][k];
            }
        } else {
            const double crx = cw * dx_ov_dt[0], cry = cw * dx_ov_dt[1];
            const double crz = cw * OR_ONE_THIRD * mom[2 * npart + p] * invgf[p];
            const int nyd = nyp + 1;
            for( int j = 0; j < 5; j++ ) {
                const double w = S0[1][j] + 0.5 * DS[1][j];
                double acc = 0.0;
                for( int i = 1; i < 5; i++ ) {
                    acc -= crx * DS[0][i - 1] * w;
                    Jx[( int64_t )( base[0] + i ) * nyp + base[1] + j] += acc;
                }
            }
            for( int i = 0; i < 5; i++ ) {
                const double w = S0[0][i] + 0.5 * DS[0][i];
                double acc = 0.0;
                for( int j = 1; j < 5; j++ ) {
                    acc -= cry * DS[1][j - 1] * w;
                    Jy[( int64_t )( base[0] + i ) * nyd + base[1] + j] += acc;
                }
            }
            for( int i = 0; i < 5; i++ )
                for( int j = 0; j < 5; j++ ) {
                    Jz[( int64_t )( base[0] + i ) * nyp + base[1] + j] +=
                        crz * ( S0[1][j] * ( 0.5 * S1[0][i] + S0[0][i] ) + S1[1][j] * ( 0.5 * S0[0][i] + S1[0][i] ) );
                    if( mode == 1 ) rho[( int64_t )( base[0] + i ) * nyp + base[1] + j] += cw * S1[0][i] * S1[1][j];
                }
        }
    }
}

/* Large particle counts are split over OpenMP threads, each depositing into a
 * private copy of the current arrays that is summed afterwards (the reference
 * gets the same effect from per-thread patches).  Small counts keep the
 * sequential order of the reference's loop. */
int or_project( int mode, int ndim, const int *n_prim, const int *domain_begin, const double *cell_length, double dt,
                int64_t npart, const double *pos, const double *mom, const double *weight, const short *charge,
                const double *invgf, const int *iold, const double *delta, double *const *J )
{
#ifdef _OPENMP
    const int nthr = omp_get_max_threads();
    if( npart >= 100000 && nthr > 1 ) {
        int64_t size[4];
        const int st[4][3] = { { 1, 0, 0 }, { 0, 1, 0 }, { 0, 0, 1 }, { 0, 0, 0 } };
        int64_t total = 0;
        for( int c = 0; c < 4; c++ ) {
            size[c] = 1;
            for( int d = 0; d < ndim; d++ ) size[c] *= n_prim[d] + st[c][d];
            if( J[c] ) total += size[c];
        }
        double *priv = calloc( ( size_t )total * nthr, sizeof( double ) );
        if( priv ) {
#pragma omp parallel num_threads( nthr )
            {
                const int t = omp_get_thread_num();
                double *Jt[4] = { NULL, NULL, NULL, NULL };
                double *base = priv + ( int64_t )t * total;
                for( int c = 0; c < 4; c++ )
                    if( J[c] ) { Jt[c] = base; base += size[c]; }
                const int64_t chunk = ( npart + nthr - 1 ) / nthr;
                const int64_t a = t * chunk, b = a + chunk < npart ? a + chunk : npart;
                if( a < b )
                    project_range( mode, ndim, n_prim, domain_begin, cell_length, dt, npart, pos, mom, weight, charge,
                                   invgf, iold, delta, Jt, a, b );
            }
            int64_t off = 0;
            for( int c = 0; c < 4; c++ ) {
                if( !J[c] ) continue;
                double *dst = J[c];
                const int64_t sc = size[c];
#pragma omp parallel for schedule( static )
                for( int64_t i = 0; i < sc; i++ ) {
                    double acc = dst[i];
                    for( int t = 0; t < nthr; t++ ) acc += priv[( int64_t )t * total + off + i];
                    dst[i] = acc;
                }
                off += sc;
            }
            free( priv );
            return 0;
        }
    }
#endif
    project_range( mode, ndim, n_prim, domain_begin, cell_length, dt, npart, pos, mom, weight, charge, invgf, iold,
                   delta, J, 0, npart );
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Yee solver on one patch's arrays.                                           */
/* Ampere MA_Solver3D_norm (MA_Solver3D_norm.cpp:18-115), all points;          */
/* 2D MA_Solver2D_norm.cpp:18-107.                                             */
/* Faraday MF_Solver3D_Yee (MF_Solver3D_Yee.cpp:18-111), interior points;      */
/* 2D MF_Solver2D_Yee.cpp:18-101.                                              */
/* F = {Ex, Ey, Ez, Bx, By, Bz, Jx, Jy, Jz}.                                   */
/* ------------------------------------------------------------------------- */
int or_maxwell_ampere( int ndim, const int *n_prim, const double *cell_length, double dt, double *const *F )
{
    double *Ex = F[0], *Ey = F[1], *Ez = F[2];
    const double *Bx = F[3], *By = F[4], *Bz = F[5], *Jx = F[6], *Jy = F[7], *Jz = F[8];
    const int nxp = n_prim[0], nyp = n_prim[1], nxd = nxp + 1, nyd = nyp + 1;
    const double dtdx = dt / cell_length[0], dtdy = dt / cell_length[1];
    if( ndim == 3 ) {
        const int nzp = n_prim[2], nzd = nzp + 1;
        const double dtdz = dt / cell_length[2];
#pragma omp parallel for schedule( static )
        for( int i = 0; i < nxd; i++ )
            for( int j = 0; j < nyp; j++ )
                for( int k = 0; k < nzp; k++ )
                    Ex[lin3( i, j, k, nyp, nzp )] += -dt * Jx[lin3( i, j, k, nyp, nzp )]
                        + dtdy * ( Bz[lin3( i, j + 1, k, nyd, nzp )] - Bz[lin3( i, j, k, nyd, nzp )] )
                        - dtdz * ( By[lin3( i, j, k + 1, nyp, nzd )] - By[lin3( i, j, k, nyp, nzd )] );
#pragma omp parallel for schedule( static )
        for( int i = 0; i < nxp; i++ )
            for( int j = 0; j < nyd; j++ )
                for( int k = 0; k < nzp; k++ )
                    Ey[lin3( i, j, k, nyd, nzp )] += -dt * Jy[lin3( i, j, k, nyd, nzp )]
                        - dtdx * ( Bz[lin3( i + 1, j, k, nyd, nzp )] - Bz[lin3( i, j, k, nyd, nzp )] )
                        + dtdz * ( Bx[lin3( i, j, k + 1, nyd, nzd )] - Bx[lin3( i, j, k, nyd, nzd )] );
#pragma omp parallel for schedule( static )
        for( int i = 0; i < nxp; i++ )
            for( int j = 0; j < nyp; j++ )
                for( int k = 0; k < nzd; k++ )
                    Ez[lin3( i, j, k, nyp, nzd )] += -dt * Jz[lin3( i, j, k, nyp, nzd )]
                        + dtdx * ( By[lin3( i + 1, j, k, nyp, nzd )] - By[lin3( i, j, k, nyp, nzd )] )
                        - dtdy * ( Bx[lin3( i, j + 1, k, nyd, nzd )] - Bx[lin3( i, j, k, nyd, nzd )] );
    } else {
        for( int x = 0; x < nxd; x++ )
            for( int y = 0; y < nyp; y++ )
                Ex[x * nyp + y] += -dt * Jx[x * nyp + y] + dtdy * ( Bz[x * nyd + y + 1] - Bz[x * nyd + y] );
        for( int x = 0; x < nxp; x++ )
            for( int y = 0; y < nyd; y++ )
                Ey[x * nyd + y] += -dt * Jy[x * nyd + y] - dtdx * ( Bz[( x + 1 ) * nyd + y] - Bz[x * nyd + y] );
        for( int x = 0; x < nxp; x++ )
            for( int y = 0; y < nyp; y++ )
                Ez[x * nyp + y] += -dt * Jz[x * nyp + y] + dtdx * ( By[( x + 1 ) * nyp + y] - By[x * nyp + y] )
                                   - dtdy * ( Bx[x * nyd + y + 1] - Bx[x * nyd + y] );
    }
    return 0;
}

/* periodic != 0: every point is computed; a point in the outermost dual layer
 * (index 0 or n_dual-1) takes the stencil of its periodic image n_cells away,
 * which is what the reference's B exchange (SyncVectorPatch::exchangeB,
 * SyncVectorPatch.cpp:667) copies into that layer of a single periodic patch.
 * periodic == 0: interior points only, exactly MF_Solver{2D,3D}_Yee. */
static inline int canon( int i, int nd, int ncell )
{
    return i == 0 ? ncell : ( i == nd - 1 ? i - ncell : i );
}

int or_maxwell_faraday( int ndim, const int *n_prim, const double *cell_length, double dt, double *const *F,
                        int periodic, const int *n_cells )
{
    const double *Ex = F[0], *Ey = F[1], *Ez = F[2];
    double *Bx = F[3], *By = F[4], *Bz = F[5];
    const int nxp = n_prim[0], nyp = n_prim[1], nxd = nxp + 1, nyd = nyp + 1;
    const double dtdx = dt / cell_length[0], dtdy = dt / cell_length[1];
    const int lo = periodic ? 0 : 1, hix = periodic ? nxd : nxd - 1, hiy = periodic ? nyd : nyd - 1;
    const int Nx = periodic ? n_cells[0] : 0, Ny = periodic ? n_cells[1] : 0;
    if( ndim == 3 ) {
        const int nzp = n_prim[2], nzd = nzp + 1;
        const double dtdz = dt / cell_length[2];
        const int hiz = periodic ? nzd : nzd - 1, Nz = periodic ? n_cells[2] : 0;
#pragma omp parallel for schedule( static )
        for( int i = 0; i < nxp; i++ )
            for( int j = lo; j < hiy; j++ )
                for( int k = lo; k < hiz; k++ ) {
                    const int jc = periodic ? canon( j, nyd, Ny ) : j, kc = periodic ? canon( k, nzd, Nz ) : k;
                    Bx[lin3( i, j, k, nyd, nzd )] += -dtdy * ( Ez[lin3( i, jc, k, nyp, nzd )] - Ez[lin3( i, jc - 1, k, nyp, nzd )] )
                        + dtdz * ( Ey[lin3( i, j, kc, nyd, nzp )] - Ey[lin3( i, j, kc - 1, nyd, nzp )] );
                }
#pragma omp parallel for schedule( static )
        for( int i = lo; i < hix; i++ )
            for( int j = 0; j < nyp; j++ )
                for( int k = lo; k < hiz; k++ ) {
                    const int ic = periodic ? canon( i, nxd, Nx ) : i, kc = periodic ? canon( k, nzd, Nz ) : k;
                    By[lin3( i, j, k, nyp, nzd )] += -dtdz * ( Ex[lin3( i, j, kc, nyp, nzp )] - Ex[lin3( i, j, kc - 1, nyp, nzp )] )
                        + dtdx * ( Ez[lin3( ic, j, k, nyp, nzd )] - Ez[lin3( ic - 1, j, k, nyp, nzd )] );
                }
#pragma omp parallel for schedule( static )
        for( int i = lo; i < hix; i++ )
            for( int j = lo; j < hiy; j++ )
                for( int k = 0; k < nzp; k++ ) {
                    const int ic = periodic ? canon( i, nxd, Nx ) : i, jc = periodic ? canon( j, nyd, Ny ) : j;
                    Bz[lin3( i, j, k, nyd, nzp )] += -dtdx * ( Ey[lin3( ic, j, k, nyd, nzp )] - Ey[lin3( ic - 1, j, k, nyd, nzp )] )
                        + dtdy * ( Ex[lin3( i, jc, k, nyp, nzp )] - Ex[lin3( i, jc - 1, k, nyp, nzp )] );
                }
    } else {
        for( int x = 0; x < nxp; x++ )
            for( int y = lo; y < hiy; y++ ) {
                const int yc = periodic ? canon( y, nyd, Ny ) : y;
                Bx[x * nyd + y] -= dtdy * ( Ez[x * nyp + yc] - Ez[x * nyp + yc - 1] );
            }
        for( int x = lo; x < hix; x++ )
            for( int y = 0; y < nyp; y++ ) {
                const int xc = periodic ? canon( x, nxd, Nx ) : x;
                By[x * nyp + y] += dtdx * ( Ez[xc * nyp + y] - Ez[( xc - 1 ) * nyp + y] );
            }
        for( int x = lo; x < hix; x++ )
            for( int y = lo; y < hiy; y++ ) {
                const int xc = periodic ? canon( x, nxd, Nx ) : x, yc = periodic ? canon( y, nyd, Ny ) : y;
                Bz[x * nyd + y] += dtdy * ( Ex[x * nyp + yc] - Ex[x * nyp + yc - 1] )
                                   - dtdx * ( Ey[xc * nyd + y] - Ey[( xc - 1 ) * nyd + y] );
            }
    }
    return 0;
}

/* ElectroMagn3D::saveMagneticFields (ElectroMagn3D.cpp:1048): B_m <- B;
 * centerMagneticFields (:1191-1239): B_m <- (B + B_m)/2.  n = points per component. */
int or_save_b( const int64_t *n, double *const *B, double *const *Bm )
{
    for( int c = 0; c < 3; c++ ) memcpy( Bm[c], B[c], ( size_t )n[c] * sizeof( double ) );
    return 0;
}

int or_center_b( const int64_t *n, double *const *B, double *const *Bm )
{
    for( int c = 0; c < 3; c++ )
        for( int64_t i = 0; i < n[c]; i++ ) Bm[c][i] = ( B[c][i] + Bm[c][i] ) * 0.5;
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Periodic ghost handling of a single patch covering the whole domain.       */
/* Fold (SyncVectorPatch::sumAllComponents, SyncVectorPatch.cpp:203-330, the   */
/* same-process branch): along each dimension in turn, the first              */
/* 1 + 2*oversize (+1 if dual) planes and their images n_cells further are     */
/* summed and both copies set to the sum.                                      */
/* dims = extents of the array, dual = per-dim dual flags.                     */
/* ------------------------------------------------------------------------- */
int or_fold_periodic( int ndim, const int *dims, const int *dual, const int *n_cells, int oversize, double *a )
{
    const int nx = dims[0], ny = dims[1], nz = ndim == 3 ? dims[2] : 1;
    for( int d = 0; d < ndim; d++ ) {
        const int g = 1 + 2 * oversize + dual[d];
        const int N = n_cells[d];
        for( int i = 0; i < nx; i++ )
            for( int j = 0; j < ny; j++ )
                for( int k = 0; k < nz; k++ ) {
                    int c = d == 0 ? i : ( d == 1 ? j : k );
                    if( c >= g ) continue;
                    int i2 = i, j2 = j, k2 = k;
                    if( d == 0 ) i2 += N; else if( d == 1 ) j2 += N; else k2 += N;
                    int64_t a1 = lin3( i, j, k, ny, nz ), a2 = lin3( i2, j2, k2, ny, nz );
                    a[a2] += a[a1];
                    a[a1] = a[a2];
                }
    }
    return 0;
}

/* Periodic particle wrap of a single patch (Patch::prepareParticles,
 * Patch.cpp:633-646): x < 0 -> x + L, x >= L -> x - L, per dimension. */
int or_wrap_positions( int ndim, const double *length, int64_t npart, double *pos )
{
    for( int d = 0; d < ndim; d++ )
        for( int64_t p = 0; p < npart; p++ ) {
            double *x = &pos[d * npart + p];
            if( *x < 0.0 ) *x += length[d];
            if( *x >= length[d] ) *x -= length[d];
        }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* One explicit PIC timestep on a single periodic patch covering the domain,  */
/* in the order of Smilei.cpp:483-747:                                         */
/*   J <- 0 (ElectroMagn::restartRhoJ, VectorPatch.cpp:4779)                   */
/*   per species: interpolate E, B_m at x^n -> push -> project J^{n+1/2}       */
/*     (Species::dynamics, Species.cpp:583-790) -> periodic wrap of x          */
/*   fold J ghosts (SyncVectorPatch::sumRhoJ)                                  */
/*   B_m <- B; Ampere; Faraday; B exchange; B_m <- (B + B_m)/2                */
/*     (VectorPatch::solveMaxwell :965-1060, finalizeSyncAndBCFields :1144)    */
/* fields: Ex Ey Ez Bx By Bz Bxm Bym Bzm Jx Jy Jz (reference layout, ghosts).  */
/* Species s: pos[s], mom[s], weight[s], charge[s], npart[s], mass[s],         */
/* pusher[s] (0 boris, 1 vay, 2 higuera-cary).                                 */
/* ------------------------------------------------------------------------- */
int or_pic_step( int ndim, const int *n_cells, int oversize, const double *cell_length, double dt, double *const *fields,
                 int nspecies, const int64_t *npart, const double *mass, const int *pusher, double *const *pos,
                 double *const *mom, double *const *weight, short *const *charge )
{
    int n_prim[3], domain_begin[3], dims[12][3];
    double dx_inv[3], length[3];
    int64_t sizes[12];
    for( int d = 0; d < 3; d++ ) {
        n_prim[d] = d < ndim ? n_cells[d] + 1 + 2 * oversize : 1;
        domain_begin[d] = d < ndim ? -oversize : 0;
        dx_inv[d] = d < ndim ? 1.0 / cell_length[d] : 0.0;
        length[d] = d < ndim ? n_cells[d] * cell_length[d] : 0.0;
    }
    /* Staggering of Ex Ey Ez Bx By Bz Bxm Bym Bzm Jx Jy Jz. */
    static const int stag[12][3] = { {1,0,0}, {0,1,0}, {0,0,1}, {0,1,1}, {1,0,1}, {1,1,0},
                                     {0,1,1}, {1,0,1}, {1,1,0}, {1,0,0}, {0,1,0}, {0,0,1} };
    for( int f = 0; f < 12; f++ ) {
        sizes[f] = 1;
        for( int d = 0; d < 3; d++ ) {
            dims[f][d] = d < ndim ? n_prim[d] + stag[f][d] : 1;
            sizes[f] *= dims[f][d];
        }
    }
    double *Jx = fields[9], *Jy = fields[10], *Jz = fields[11];
    for( int f = 9; f < 12; f++ ) memset( fields[f], 0, ( size_t )sizes[f] * sizeof( double ) );
    const double *gfields[6] = { fields[0], fields[1], fields[2], fields[6], fields[7], fields[8] };
    for( int s = 0; s < nspecies; s++ ) {
        const int64_t n = npart[s];
        if( n == 0 ) continue;
        double *Epart = malloc( 3 * n * sizeof( double ) ), *Bpart = malloc( 3 * n * sizeof( double ) );
        double *delta = malloc( ndim * n * sizeof( double ) ), *invgf = malloc( n * sizeof( double ) );
        int *iold = malloc( ndim * n * sizeof( int ) );
        or_interpolate( ndim, n_prim, domain_begin, dx_inv, gfields, n, pos[s], Epart, Bpart, iold, delta );
        or_push( pusher[s], ndim, dt, mass[s], n, pos[s], mom[s], charge[s], Epart, Bpart, invgf );
        double *J[4] = { Jx, Jy, Jz, NULL };
        or_project( 0, ndim, n_prim, domain_begin, cell_length, dt, n, pos[s], mom[s], weight[s], charge[s], invgf, iold, delta, J );
        or_wrap_positions( ndim, length, n, pos[s] );
        free( Epart ); free( Bpart ); free( delta ); free( invgf ); free( iold );
    }
    for( int f = 9; f < 12; f++ ) {
        int dual[3] = { stag[f][0], stag[f][1], stag[f][2] };
        or_fold_periodic( ndim, dims[f], dual, n_cells, oversize, fields[f] );
    }
    double *B[3] = { fields[3], fields[4], fields[5] }, *Bm[3] = { fields[6], fields[7], fields[8] };
    or_save_b( &sizes[3], B, Bm );
    double *F[9] = { fields[0], fields[1], fields[2], fields[3], fields[4], fields[5], Jx, Jy, Jz };
    or_maxwell_ampere( ndim, n_prim, cell_length, dt, F );
    or_maxwell_faraday( ndim, n_prim, cell_length, dt, F, 1, n_cells );
    or_center_b( &sizes[3], B, Bm );
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Per-cell particle sort (SpeciesV::computeParticleCellKeys,                 */
/* SpeciesV.cpp:766-857, and the counts / first_index / last_index prefix sum */
/* of SpeciesV::sortParticles :599-660).                                      */
/* key = sum_d (round(x_d/dx_d) - round(xmin_d/dx_d)) * stride_d over the      */
/* (patch_size+1)^ndim node lattice.  Produces a stable permutation (original */
/* order kept inside a cell; the reference's cycle sort fixes the bins and    */
/* their members but not the order inside a bin).                            */
/* ------------------------------------------------------------------------- */
int or_sort_keys( int ndim, const int *patch_size, const double *xmin, const double *dx_inv, int64_t npart,
                  const double *pos, int *keys )
{
    double mn[3];
    for( int d = 0; d < ndim; d++ ) mn[d] = round( xmin[d] * dx_inv[d] );
    for( int64_t p = 0; p < npart; p++ ) {
        int key = 0;
        for( int d = 0; d < ndim; d++ ) {
            key *= ( patch_size[d] + 1 );
            key += ( int )( round( pos[d * npart + p] * dx_inv[d] ) - mn[d] );
        }
        keys[p] = key;
    }
    return 0;
}

int or_sort_bins( int64_t npart, const int *keys, int ncell, int *first_index, int *last_index, int64_t *perm )
{
    int64_t *count = calloc( ( size_t )ncell + 1, sizeof( int64_t ) );
    for( int64_t p = 0; p < npart; p++ ) count[keys[p]]++;
    int64_t run = 0;
    for( int c = 0; c < ncell; c++ ) {
        first_index[c] = ( int )run;
        run += count[c];
        last_index[c] = ( int )run;
    }
    int64_t *fill = calloc( ( size_t )ncell + 1, sizeof( int64_t ) );
    for( int c = 0; c < ncell; c++ ) fill[c] = first_index[c];
    for( int64_t p = 0; p < npart; p++ ) perm[fill[keys[p]]++] = p;
    free( count );
    free( fill );
    return 0;
}
