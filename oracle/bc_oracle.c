/* CPU restatement of the reference's open boundaries in 2D -- TEST INFRASTRUCTURE ONLY.
 *
 * Silver-Mueller field boundaries with laser injection, particle removal at
 * non-periodic boundaries, and a 2D timestep that uses them.  Only tests/,
 * the smoke check and the benchmark's CPU legs load this code; the product
 * path is the CUDA library.  Every function cites the reference file:line it
 * follows.
 *
 * Field layout as in pic_oracle.c: reference arrays with ghost width 2,
 * F = {Ex, Ey, Ez, Bx, By, Bz} (2D: index x * ny + y with the component's own
 * ny, primal or dual).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* pic_oracle.c */
int or_interpolate( int ndim, const int *n_prim, const int *domain_begin, const double *dx_inv,
                    const double *const *fields, int64_t npart, const double *pos, double *Epart, double *Bpart,
                    int *iold, double *delta );
int or_push( int kind, int ndim, double dt, double mass, int64_t npart, double *pos, double *mom, const short *charge,
             const double *Epart, const double *Bpart, double *invgf );
int or_project( int mode, int ndim, const int *n_prim, const int *domain_begin, const double *cell_length, double dt,
                int64_t npart, const double *pos, const double *mom, const double *weight, const short *charge,
                const double *invgf, const int *iold, const double *delta, double *const *J );
int or_maxwell_ampere( int ndim, const int *n_prim, const double *cell_length, double dt, double *const *F );
int or_save_b( const int64_t *n, double *const *B, double *const *Bm );
int or_center_b( const int64_t *n, double *const *B, double *const *Bm );
int or_fold_periodic( int ndim, const int *dims, const int *dual, const int *n_cells, int oversize, double *a );

/* ------------------------------------------------------------------------- */
/* Silver-Mueller coefficients of one side (ElectroMagnBC2D_SM constructor,   */
/* src/ElectroMagnBC/ElectroMagnBC2D_SM.cpp:18-66).  side = 2*axis + (max?1:0); */
/* k = incoming wave vector of that side (default: +-unit normal, inward,     */
/* Params.cpp:476-493).  c = {Alpha, Beta, Gamma, Delta, Epsilon}.            */
/* ------------------------------------------------------------------------- */
int or_sm_coefficients( int side, const double *cell_length, double dt, const double *k, double *c )
{
    const int a0 = side / 2, a1 = a0 == 0 ? 1 : 0;
    const double sgn = ( double )( side % 2 ) * 2.0 - 1.0;
    const double kn = sqrt( k[0] * k[0] + k[1] * k[1] );
    const double k0 = k[a0] / kn, k1 = k[a1] / kn;
    const double dt0 = dt / cell_length[a0], dt1 = dt / cell_length[a1];
    const double factor = 1.0 / ( k0 - sgn * dt0 );
    c[0] = 2.0 * factor;
    c[1] = -( k0 + sgn * dt0 ) * factor;
    c[2] = 4.0 * k0 * factor;
    c[3] = -( k1 + dt1 ) * factor;
    c[4] = -( k1 - dt1 ) * factor;
    return 0;
}

/* ------------------------------------------------------------------------- */
/* One side of the 2D Silver-Mueller condition, without external fields      */
/* (ElectroMagnBC2D_SM::apply, ElectroMagnBC2D_SM.cpp:118-265).  b1: incoming */
/* amplitudes on the primal points along the side (n_prim of the tangent      */
/* axis), b2 on the dual points; NULL = no laser.  tmin/tmax: whether the     */
/* tangent axis ends are boundaries (then its first / last point is skipped). */
/* ------------------------------------------------------------------------- */
int or_sm_apply_2d( int side, const int *n_prim, const double *cell_length, double dt, const double *k,
                    double *const *F, const double *b1, const double *b2, int tmin, int tmax )
{
    const double *Ex = F[0], *Ey = F[1], *Ez = F[2];
    double *Bx = F[3], *By = F[4], *Bz = F[5];
    double c[5];
    or_sm_coefficients( side, cell_length, dt, k, c );
    const double Al = c[0], Be = c[1], Ga = c[2], De = c[3], Ep = c[4];
    const int a0 = side / 2, a1 = a0 == 0 ? 1 : 0;
    const int mx = side % 2;
    const int sgn = mx ? 1 : -1;
    const int np0 = n_prim[a0], nd0 = np0 + 1;
    const int nyp = n_prim[1], nyd = nyp + 1;
    int iB[3];
    if( !mx ) {
        iB[0] = iB[1] = iB[2] = 0;
    } else {
        iB[a0] = np0 - 1;
        iB[a1] = nd0 - 1;
        iB[2] = nd0 - 1;
    }
    const int p0 = iB[0] - sgn, p1 = iB[1] - sgn, p2 = iB[2] - sgn;
    const int n1p = n_prim[a1], n1d = n1p + 1;
    if( a0 == 0 ) {
        for( int j = tmin; j < n1p - tmax; j++ ) /* By (d,p) */
            By[iB[1] * nyp + j] = Al * Ez[iB[0] * nyp + j] + Be * By[p1 * nyp + j] + Ga * ( b1 ? b1[j] : 0.0 )
                                  + De * Bx[iB[0] * nyd + j + 1] + Ep * Bx[iB[0] * nyd + j];
        for( int j = tmin; j < n1d - tmax; j++ ) /* Bz (d,d) */
            Bz[iB[2] * nyd + j] = -Al * Ey[iB[0] * nyd + j] + Be * Bz[p2 * nyd + j] + Ga * ( b2 ? b2[j] : 0.0 );
    } else {
        for( int j = tmin; j < n1p - tmax; j++ ) /* Bx (p,d) */
            Bx[iB[0] + nyd * j] = -Al * Ez[iB[1] + nyp * j] + Be * Bx[p0 + nyd * j] + Ga * ( b1 ? b1[j] : 0.0 )
                                  + De * By[iB[1] + nyp * ( j + 1 )] + Ep * By[iB[1] + nyp * j];
        for( int j = tmin; j < n1d - tmax; j++ ) /* Bz (d,d) */
            Bz[j * nyd + iB[2]] = Al * Ex[j * nyp + iB[1]] + Be * Bz[j * nyd + p2] + Ga * ( b2 ? b2[j] : 0.0 );
    }
    (void)nd0;
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Gaussian 2D laser at an x side (pyprofiles.py LaserGaussian2D :507-569,    */
/* without incidence angle; transformPolarization :458-468; tgaussian         */
/* :334-353 as compiled, Function.cpp:528-535) and its separable amplitude    */
/* (LaserProfileSeparable::getAmplitude, Laser.cpp:453-460):                  */
/*   amp_p(y, t) = T(t - (phi_p(y) + delay_p) / omega) S_p(y) sin(omega t - phi_p(y)) */
/* p = 0: the profile on the primal points (By), p = 1: on the dual points (Bz). */
/* prm: {a0, omega, waist, focus_x, focus_y, polarization_phi, ellipticity,     */
/*       phase_offset, t_start, t_duration, t_center, t_fwhm, t_order, side_max} */
/* (focus_x as given by the user; for a max side the distance is grid_length_x */
/* minus it, passed already converted).                                       */
/* ------------------------------------------------------------------------- */
static double tgaussian( const double *prm, double t )
{
    const double start = prm[8], end = prm[8] + prm[9], center = prm[10], fwhm = prm[11], order = prm[12];
    const double sigma = pow( 0.5 * fwhm, order ) / log( 2.0 );
    if( t < start || t > end ) return 0.0;
    return exp( -pow( t - center, order ) * ( 1.0 / sigma ) );
}

int or_laser_gaussian2d( const double *prm, int n, const double *y, int profile, double t, double *out )
{
    const double a0 = prm[0], omega = prm[1], waist = prm[2], fx = prm[3], fy = prm[4];
    const double pphi = prm[5], ell = prm[6], phase_offset = prm[7];
    /* transformPolarization */
    const double e2 = ell * ell;
    const double pp = ( 1.0 - e2 ) * sin( 2.0 * pphi ) / 2.0;
    const double dephasing = atan2( ell, pp );
    const double amplitude = sqrt( 1.0 / ( 1.0 + e2 ) );
    const double c2 = cos( pphi ) * cos( pphi ), s2 = 1.0 - c2;
    /* LaserGaussian2D unpacks transformPolarization's [dephasing, A1, A2] as
       (dephasing, amplitudeZ, amplitudeY): profile 0 (By) takes A2, profile 1 (Bz) A1 */
    const double ampY = amplitude * sqrt( s2 + e2 * c2 ) * a0 * omega;
    const double ampZ = amplitude * sqrt( c2 + e2 * s2 ) * a0 * omega;
    const double delay[2] = { 0.0, dephasing };
    const double Zr = omega * waist * waist / 2.0;
    const double w = sqrt( 1.0 / ( 1.0 + ( fx / Zr ) * ( fx / Zr ) ) );
    const double invWaist2 = ( w / waist ) * ( w / waist );
    const double coeff = -omega * fx * w * w / ( 2.0 * Zr * Zr );
    for( int j = 0; j < n; j++ ) {
        const double dy = y[j] - fy;
        const double spatial = sqrt( w ) * exp( -invWaist2 * dy * dy );
        const double ph = coeff * dy * dy;
        /* profile 0: space ampY * spatial, phase ph - offset + delay[1], delay delay[0];
           profile 1: space ampZ * spatial, phase ph - offset + delay[0], delay delay[1] */
        const double S = profile == 0 ? ampY * spatial : ampZ * spatial;
        const double phi = ph - phase_offset + ( profile == 0 ? delay[1] : delay[0] );
        const double dl = profile == 0 ? delay[0] : delay[1];
        out[j] = tgaussian( prm, t - ( phi + dl ) / omega ) * S * sin( omega * t - phi );
    }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Faraday with per-dimension periodicity (MF_Solver2D_Yee::operator(),       */
/* src/ElectroMagnSolver/MF_Solver2D_Yee.cpp:18-140): interior points along a */
/* non-periodic axis (left to the boundary condition), all points along a     */
/* periodic one with the outermost dual layer taken from its periodic image.  */
/* ------------------------------------------------------------------------- */
static inline int canon( int i, int nd, int ncell )
{
    return i == 0 ? ncell : ( i == nd - 1 ? i - ncell : i );
}

int or_faraday_2d( const int *n_prim, const double *cell_length, double dt, double *const *F, const int *periodic,
                   const int *n_cells )
{
    const double *Ex = F[0], *Ey = F[1], *Ez = F[2];
    double *Bx = F[3], *By = F[4], *Bz = F[5];
    const int nxp = n_prim[0], nyp = n_prim[1], nxd = nxp + 1, nyd = nyp + 1;
    const double dtdx = dt / cell_length[0], dtdy = dt / cell_length[1];
    const int lox = periodic[0] ? 0 : 1, hix = periodic[0] ? nxd : nxd - 1;
    const int loy = periodic[1] ? 0 : 1, hiy = periodic[1] ? nyd : nyd - 1;
    for( int x = 0; x < nxp; x++ )
        for( int y = loy; y < hiy; y++ ) {
            const int yc = periodic[1] ? canon( y, nyd, n_cells[1] ) : y;
            Bx[x * nyd + y] -= dtdy * ( Ez[x * nyp + yc] - Ez[x * nyp + yc - 1] );
        }
    for( int x = lox; x < hix; x++ )
        for( int y = 0; y < nyp; y++ ) {
            const int xc = periodic[0] ? canon( x, nxd, n_cells[0] ) : x;
            By[x * nyp + y] += dtdx * ( Ez[xc * nyp + y] - Ez[( xc - 1 ) * nyp + y] );
        }
    for( int x = lox; x < hix; x++ )
        for( int y = loy; y < hiy; y++ ) {
            const int xc = periodic[0] ? canon( x, nxd, n_cells[0] ) : x, yc = periodic[1] ? canon( y, nyd, n_cells[1] ) : y;
            Bz[x * nyd + y] += dtdy * ( Ex[x * nyp + yc] - Ex[x * nyp + yc - 1] ) - dtdx * ( Ey[xc * nyd + y] - Ey[( xc - 1 ) * nyd + y] );
        }
    return 0;
}

/* Fold of the J ghosts along the periodic dimensions only (the same-process
 * branch of SyncVectorPatch::sumAllComponents, SyncVectorPatch.cpp:203-330):
 * planes 0 .. 2*oversize (+1 if dual) and their images n_cells further are
 * summed and both set to the sum. */
static void fold_dims( const int *dims, const int *dual, const int *n_cells, int oversize, const int *periodic, double *a )
{
    const int nx = dims[0], ny = dims[1];
    for( int d = 0; d < 2; d++ ) {
        if( !periodic[d] ) continue;
        const int g = 1 + 2 * oversize + dual[d], N = n_cells[d];
        for( int i = 0; i < nx; i++ )
            for( int j = 0; j < ny; j++ ) {
                const int c = d == 0 ? i : j;
                if( c >= g ) continue;
                const int64_t a1 = ( int64_t )i * ny + j, a2 = d == 0 ? ( int64_t )( i + N ) * ny + j : ( int64_t )i * ny + j + N;
                a[a2] += a[a1];
                a[a1] = a[a2];
            }
    }
}

/* ------------------------------------------------------------------------- */
/* One 2D timestep with open boundaries (Smilei.cpp:483-747 order):           */
/*   J <- 0; per species: interpolate, push, then along a non-periodic axis a */
/*   particle at x < 0 or x >= L gets charge 0 (remove_particle_inf/_sup,     */
/*   src/ParticleBC/BoundaryConditionType.cpp:204-294) so it deposits no      */
/*   current, project J, wrap the periodic axes, drop the removed particles   */
/*   (order kept); fold J along the periodic axes; B_m <- B; Ampere (all      */
/*   points); Faraday (interior along open axes); Silver-Mueller on the open  */
/*   sides in the order xmin, xmax, ymin, ymax (ElectroMagn::boundaryConditions, */
/*   ElectroMagn.cpp:371-394) with the laser of `laser` (NULL: none) on xmin  */
/*   at time_dual; B_m <- (B + B_m)/2.                                        */
/* skip_x: the moving window shifts at the end of this step, so the x sides  */
/*   are skipped (ElectroMagn.cpp:374, SimWindow::isMoving).                  */
/* npart[s] is updated; the arrays of species s are compacted in place.      */
/* ------------------------------------------------------------------------- */
int or_pic_step_bc( const int *n_cells, int oversize, const double *cell_length, double dt, double *const *fields,
                    int nspecies, int64_t *npart, const double *mass, const int *pusher, double *const *pos,
                    double *const *mom, double *const *weight, short *const *charge, const int *periodic,
                    const double *laser, double time_dual, int skip_x )
{
    const int ndim = 2;
    int n_prim[3], domain_begin[3], dims[12][3];
    double dx_inv[3], length[3];
    int64_t sizes[12];
    for( int d = 0; d < 3; d++ ) {
        n_prim[d] = d < ndim ? n_cells[d] + 1 + 2 * oversize : 1;
        domain_begin[d] = d < ndim ? -oversize : 0;
        dx_inv[d] = d < ndim ? 1.0 / cell_length[d] : 0.0;
        length[d] = d < ndim ? n_cells[d] * cell_length[d] : 0.0;
    }
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
        char *gone = calloc( ( size_t )n, 1 );
        for( int d = 0; d < ndim; d++ ) {
            if( periodic[d] ) continue;
            for( int64_t p = 0; p < n; p++ ) {
                const double x = pos[s][d * n + p];
                if( x < 0.0 || x >= length[d] ) {
                    charge[s][p] = 0;
                    gone[p] = 1;
                }
            }
        }
        double *J[4] = { Jx, Jy, Jz, NULL };
        or_project( 0, ndim, n_prim, domain_begin, cell_length, dt, n, pos[s], mom[s], weight[s], charge[s], invgf, iold, delta, J );
        for( int d = 0; d < ndim; d++ ) {
            if( !periodic[d] ) continue;
            for( int64_t p = 0; p < n; p++ ) {
                double *x = &pos[s][d * n + p];
                if( *x < 0.0 ) *x += length[d];
                if( *x >= length[d] ) *x -= length[d];
            }
        }
        int64_t m = 0;
        for( int64_t p = 0; p < n; p++ ) {
            if( gone[p] ) continue;
            for( int d = 0; d < ndim; d++ ) pos[s][d * n + m] = pos[s][d * n + p];
            for( int c = 0; c < 3; c++ ) mom[s][c * n + m] = mom[s][c * n + p];
            weight[s][m] = weight[s][p];
            charge[s][m] = charge[s][p];
            m++;
        }
        /* close the gaps of the component planes (planes of n -> planes of m) */
        for( int d = 1; d < ndim; d++ ) memmove( &pos[s][d * m], &pos[s][d * n], ( size_t )m * sizeof( double ) );
        for( int c = 1; c < 3; c++ ) memmove( &mom[s][c * m], &mom[s][c * n], ( size_t )m * sizeof( double ) );
        npart[s] = m;
        free( gone ); free( Epart ); free( Bpart ); free( delta ); free( invgf ); free( iold );
    }
    for( int f = 9; f < 12; f++ ) {
        int dual[3] = { stag[f][0], stag[f][1], stag[f][2] };
        fold_dims( dims[f], dual, n_cells, oversize, periodic, fields[f] );
    }
    double *B[3] = { fields[3], fields[4], fields[5] }, *Bm[3] = { fields[6], fields[7], fields[8] };
    or_save_b( &sizes[3], B, Bm );
    double *F[9] = { fields[0], fields[1], fields[2], fields[3], fields[4], fields[5], Jx, Jy, Jz };
    or_maxwell_ampere( ndim, n_prim, cell_length, dt, F );
    or_faraday_2d( n_prim, cell_length, dt, F, periodic, n_cells );
    static const double kdef[4][2] = { { 1.0, 0.0 }, { -1.0, 0.0 }, { 0.0, 1.0 }, { 0.0, -1.0 } };
    for( int side = 0; side < 4; side++ ) {
        const int ax = side / 2, tan = ax == 0 ? 1 : 0;
        if( periodic[ax] || ( ax == 0 && skip_x ) ) continue;
        double *b1 = NULL, *b2 = NULL;
        if( side == 0 && laser ) {
            const int n1p = n_prim[1], n1d = n1p + 1;
            double *y = malloc( ( size_t )n1d * sizeof( double ) );
            b1 = calloc( ( size_t )n1p, sizeof( double ) );
            b2 = calloc( ( size_t )n1d, sizeof( double ) );
            for( int j = 0; j < n1p; j++ ) y[j] = ( j - oversize ) * cell_length[1];
            or_laser_gaussian2d( laser, n1p, y, 0, time_dual, b1 );
            for( int j = 0; j < n1d; j++ ) y[j] = ( j - 0.5 - oversize ) * cell_length[1];
            or_laser_gaussian2d( laser, n1d, y, 1, time_dual, b2 );
            free( y );
        }
        or_sm_apply_2d( side, n_prim, cell_length, dt, kdef[side], F, b1, b2, !periodic[tan], !periodic[tan] );
        free( b1 );
        free( b2 );
    }
    or_center_b( &sizes[3], B, Bm );
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Moving window on one grid (SimWindow::shift, src/MovWindow/SimWindow.cpp:  */
/* 98-560).  The reference drops its xmin patch and appends a fresh patch at   */
/* xmax: fields of the fresh patch start at zero, the particles of the dropped */
/* patch are lost, and particles keep absolute positions while the grid origin */
/* advances by `shift` cells.  Here the grid stays put and its contents move:  */
/* a point at window index i takes the value of point i + shift when it lies   */
/* in front of the fresh region (position < (N - shift) dx), else 0; primal    */
/* index i sits at (i - oversize) dx, dual at (i - oversize - 1/2) dx along x. */
/* All 12 arrays (E, B, B_m, J) move.                                          */
/* ------------------------------------------------------------------------- */
int or_window_shift_fields( int ndim, const int *n_cells, int oversize, int shift, double *const *fields )
{
    static const int stag[12][3] = { {1,0,0}, {0,1,0}, {0,0,1}, {0,1,1}, {1,0,1}, {1,1,0},
                                     {0,1,1}, {1,0,1}, {1,1,0}, {1,0,0}, {0,1,0}, {0,0,1} };
    if( shift <= 0 || shift > n_cells[0] ) return -1;
    for( int f = 0; f < 12; f++ ) {
        int64_t dims[3];
        for( int d = 0; d < 3; d++ ) dims[d] = d < ndim ? n_cells[d] + 1 + 2 * oversize + stag[f][d] : 1;
        const int64_t plane = dims[1] * dims[2];
        const int64_t keep = ( int64_t )n_cells[0] - shift + oversize + stag[f][0]; /* first index of the fresh region */
        double *a = fields[f];
        for( int64_t i = 0; i < dims[0]; i++ )
            for( int64_t t = 0; t < plane; t++ )
                a[i * plane + t] = i < keep ? a[( i + shift ) * plane + t] : 0.0;
    }
    return 0;
}

/* Particles of one species follow the window: x -= shift dx (the FP64 form keeps  */
/* window positions; the reference keeps absolute ones and moves the origin), and */
/* a particle now at x < 0 was in the dropped patch and is removed.  The arrays   */
/* are compacted in place, order kept; returns the survivors' count.              */
int64_t or_window_shift_particles( int ndim, double dx, int shift, int64_t n, double *pos, double *mom, double *weight,
                                   short *charge )
{
    const double sx = ( double )shift * dx;
    int64_t m = 0;
    for( int64_t p = 0; p < n; p++ ) {
        const double x = pos[p] - sx;
        if( x < 0.0 ) continue;
        pos[m] = x;
        for( int d = 1; d < ndim; d++ ) pos[d * n + m] = pos[d * n + p];
        for( int c = 0; c < 3; c++ ) mom[c * n + m] = mom[c * n + p];
        weight[m] = weight[p];
        if( charge ) charge[m] = charge[p];
        m++;
    }
    for( int d = 1; d < ndim; d++ ) memmove( &pos[d * m], &pos[d * n], ( size_t )m * sizeof( double ) );
    for( int c = 1; c < 3; c++ ) memmove( &mom[c * m], &mom[c * n], ( size_t )m * sizeof( double ) );
    return m;
}

/* Trapezoidal profile (trapeze, src/Profiles/Function.cpp:291-310). */
static double trapeze( double x, double plateau, double slope1, double slope2 )
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

/* Counter-based random numbers for the momenta of created particles: the     */
/* splitmix64 output function (Steele, Lea and Flood 2014, as published by    */
/* Vigna) applied to a key built from (seed, absolute cell, particle, draw).   */
/* Not the reference's generator: the reference draws from one stream per      */
/* patch; a counter-based key makes every particle's draw independent of the   */
/* order of creation, which is what a parallel creator needs.                  */
static inline uint64_t mix64( uint64_t z )
{
    z += 0x9E3779B97F4A7C15ull;
    z = ( z ^ ( z >> 30 ) ) * 0xBF58476D1CE4E5B9ull;
    z = ( z ^ ( z >> 27 ) ) * 0x94D049BB133111EBull;
    return z ^ ( z >> 31 );
}

static inline double uniform_open0( uint64_t seed, uint64_t cell, uint64_t k )
{
    const uint64_t h = mix64( mix64( seed ^ mix64( cell ) ) + k );
    return ( double )( ( h >> 11 ) + 1 ) * ( 1.0 / 9007199254740992.0 ); /* (0, 1] */
}

/* Particle creation in window cells [x0, x1) x all y (x all z), regular       */
/* positions (ParticleCreator::create and createPosition, src/Particles/        */
/* ParticleCreator.cpp:110-345, 615-667): ppc = c^ndim particles per cell where */
/* the density is non-zero, at x = i dx + dx 0.975 / c (0.5 + m), m the          */
/* particle's index along x (fastest), then y, z; weight = n(x_centre) dx dy    */
/* (dz) / ppc (createWeight, :933-939) with n evaluated at the absolute cell    */
/* centre (n_moved + i + 1/2) dx of a trapezoidal profile in x;                  */
/* prof = {n0, x_vacuum, x_slope1, x_plateau, x_slope2}.  Momenta: zero when     */
/* temperature == 0, else sqrt(temperature) times standard normals (Box-Muller), */
/* the non-relativistic limit of the reference's Maxwell-Juettner sampling.      */
/* Cells x-major, then y, z; returns the number created (at most cap; -1 when   */
/* cap is too small or ppc is not a power ndim).                                 */
int64_t or_create_particles( int ndim, const int *n_cells, const double *cell_length, int x0, int x1,
                             int64_t n_moved, const double *prof, int ppc, double temperature, uint64_t seed,
                             double *pos, double *mom, double *weight, int64_t cap )
{
    int c = 1;
    while( ( ndim == 2 ? c * c : c * c * c ) < ppc ) c++;
    if( ( ndim == 2 ? c * c : c * c * c ) != ppc ) return -1;
    const double invc = 1.0 / ( double )c;
    const int ny = n_cells[1], nz = ndim == 3 ? n_cells[2] : 1;
    double vol = 1.0;
    for( int d = 0; d < ndim; d++ ) vol *= cell_length[d];
    const double sq = sqrt( temperature );
    int64_t n = 0;
    for( int i = x0; i < x1; i++ ) {
        const double xc = ( ( double )( n_moved + i ) + 0.5 ) * cell_length[0];
        const double dens = prof[0] * trapeze( xc - prof[1], prof[3], prof[2], prof[4] );
        if( !( dens > 0.0 ) ) continue;
        const double w = dens * vol / ( double )ppc;
        for( int j = 0; j < ny; j++ )
            for( int k = 0; k < nz; k++ ) {
                const int ci[3] = { i, j, k };
                const uint64_t cell = ( ( uint64_t )( n_moved + i ) * ( uint64_t )ny + ( uint64_t )j ) * ( uint64_t )nz + ( uint64_t )k;
                for( int p = 0; p < ppc; p++ ) {
                    if( n >= cap ) return -1;
                    int m = p;
                    for( int d = 0; d < ndim; d++ ) {
                        pos[d * cap + n] = ( double )ci[d] * cell_length[d] + cell_length[d] * 0.975 * invc * ( 0.5 + ( double )( m % c ) );
                        m /= c;
                    }
                    for( int q = 0; q < 3; q++ ) mom[q * cap + n] = 0.0;
                    if( temperature > 0.0 ) {
                        const uint64_t base = ( uint64_t )p * 4u;
                        const double r1 = sqrt( -2.0 * log( uniform_open0( seed, cell, base ) ) );
                        const double a1 = 6.283185307179586 * uniform_open0( seed, cell, base + 1 );
                        const double r2 = sqrt( -2.0 * log( uniform_open0( seed, cell, base + 2 ) ) );
                        const double a2 = 6.283185307179586 * uniform_open0( seed, cell, base + 3 );
                        mom[n] = sq * r1 * cos( a1 );
                        mom[cap + n] = sq * r1 * sin( a1 );
                        mom[2 * cap + n] = sq * r2 * cos( a2 );
                    }
                    weight[n] = w;
                    n++;
                }
            }
    }
    return n;
}
