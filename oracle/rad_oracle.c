/* rad_oracle.c -- CPU restatement of the reference's Monte-Carlo radiation reaction.
 *
 * TEST INFRASTRUCTURE ONLY (see pic_oracle.c).  FP64, the reference's table
 * conventions (src/Radiation/Table.cpp:77-110: log10_min = log10(min),
 * delta = (log10(max) - log10_min)/(size-1), inv_delta = 1/delta).
 *
 * The per-particle random stream is counter based so that the GPU kernel and
 * this oracle draw identical numbers: state = fmix32(seed ^ fmix32(id) ^
 * fmix32(step + 0x9e3779b9)) (MurmurHash3's 32-bit finaliser), then
 * successive xorshift32 steps (Marsaglia 2003, as src/Tools/Random.h:9-20),
 * each mapped to (0, 1) by x / 2^32 (Random::uniform, Random.h:74-75,129, the
 * draw RadiationMonteCarlo::operator() makes).  A reference Random seeded with
 * a particle's initial state draws that particle's stream.
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>

static inline uint32_t fmix32( uint32_t h )
{
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}

static inline uint32_t xorshift32( uint32_t s )
{
    s ^= s << 13;
    s ^= s >> 17;
    s ^= s << 5;
    return s;
}

uint32_t or_rng_init( uint32_t seed, uint32_t id, uint32_t step )
{
    uint32_t s = fmix32( seed ^ fmix32( id ) ^ fmix32( step + 0x9e3779b9u ) );
    return s ? s : 0xffffffffu;
}

static inline double rng_uniform( uint32_t *s )
{
    *s = xorshift32( *s );
    return ( double )( *s ) * ( 1.0 / 4294967296.0 );
}

typedef struct {
    const double *integ;
    int n_integ;
    double integ_log10_min, integ_delta, integ_inv_delta;
    const double *xi;
    int n_chi, n_ph;
    double xi_log10_min, xi_delta, xi_inv_delta, inv_nph_m1;
    const double *axis1_min;
    double factor_dNph_dt;          /* sqrt(3) alpha / (2 pi lambda_C) (RadiationTables.cpp:99) */
    double factor_classical;        /* 2 alpha / (3 lambda_C) (RadiationTables.cpp:102) */
    double min_chi_continuous;      /* 1e-3 by default */
    double min_chi_discontinuous;   /* 1e-2 by default */
    double inv_norm_E_schwinger;    /* hbar omega_r / (m c^2) (Radiation.cpp:29-33) */
} or_rad_tables;

/* userFunctions::searchValuesInMonotonicArray (src/Tools/userFunctions.h:248-272) */
static int search_monotonic( const double *a, double v, int n )
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

/* RadiationTables::computePhotonProductionYield (RadiationTables.cpp:225-262) */
double or_rad_yield( const or_rad_tables *t, double chi, double gamma )
{
    const double lc = log10( chi );
    int i = ( int )floor( ( lc - t->integ_log10_min ) * t->integ_inv_delta );
    double v;
    if( i < 0 ) {
        v = t->integ[0];
    } else if( i >= t->n_integ - 1 ) {
        v = t->integ[t->n_integ - 2];
    } else {
        const double lm = i * t->integ_delta + t->integ_log10_min, lp = lm + t->integ_delta;
        v = ( t->integ[i + 1] * fabs( lc - lm ) + t->integ[i] * fabs( lp - lc ) ) * t->integ_inv_delta;
    }
    return t->factor_dNph_dt * v * chi / gamma;
}

/* RadiationTables::computeRandomPhotonChiWithInterpolation (RadiationTables.cpp:375-512) */
double or_rad_photon_chi( const or_rad_tables *t, double chi, double xi )
{
    const int n1 = t->n_ph;
    const double lc = log10( chi );
    int ic = ( int )floor( ( lc - t->xi_log10_min ) * t->xi_inv_delta );
    if( ic < 0 ) ic = 0;
    else if( ic > t->n_chi - 2 ) ic = t->n_chi - 2;
    int i1, i2;
    if( xi <= t->xi[ic * n1] ) {
        i1 = 0;
        i2 = 0;
        xi = t->xi[ic * n1];
    } else {
        i1 = search_monotonic( &t->xi[ic * n1], xi, n1 );
        i2 = search_monotonic( &t->xi[( ic + 1 ) * n1], xi, n1 );
    }
    const double dchi = ( lc - ( ic * t->xi_delta + t->xi_log10_min ) ) * t->xi_inv_delta;
    const double d1 = ( ic * t->xi_delta + t->xi_log10_min - t->axis1_min[ic] ) * t->inv_nph_m1;
    const double d2 = ( ( ic + 1 ) * t->xi_delta + t->xi_log10_min - t->axis1_min[ic + 1] ) * t->inv_nph_m1;
    const int x1 = ic * n1 + i1, x2 = ( ic + 1 ) * n1 + i2;
    double p1, p2;
    if( t->xi[x1] < 1.0 && t->xi[x1 + 1] - t->xi[x1] > 1e-15 ) {
        const double lm = i1 * d1 + t->axis1_min[ic], lp = lm + d1;
        const double d = ( xi - t->xi[x1] ) / ( t->xi[x1 + 1] - t->xi[x1] );
        p1 = lm * ( 1.0 - d ) + lp * d;
    } else {
        p1 = i1 * d1 + t->axis1_min[ic];
    }
    if( t->xi[x2] < 1.0 && t->xi[x2 + 1] - t->xi[x2] > 1e-15 ) {
        const double lm = i2 * d2 + t->axis1_min[ic + 1], lp = lm + d2;
        const double d = ( xi - t->xi[x2] ) / ( t->xi[x2 + 1] - t->xi[x2] );
        p2 = lm * ( 1.0 - d ) + lp * d;
    } else {
        p2 = i2 * d2 + t->axis1_min[ic + 1];
    }
    return pow( 10.0, p1 * ( 1 - dchi ) + p2 * dchi );
}

/* Radiation::computeParticleChi (Radiation.h:71-83) */
static inline double particle_chi( double qm2, double px, double py, double pz, double g, double Ex, double Ey,
                                   double Ez, double Bx, double By, double Bz, double inv_es )
{
    const double a = Ex * px + Ey * py + Ez * pz;
    const double b = g * Ex - By * pz + Bz * py;
    const double c = g * Ey - Bz * px + Bx * pz;
    const double d = g * Ez - Bx * py + By * px;
    return fabs( qm2 ) * inv_es * sqrt( fabs( a * a - b * b - c * c - d * d ) );
}

/* RadiationTables::computeRidgersFit / getRidgersCorrectedRadiatedEnergy (RadiationTables.h) */
static inline double ridgers_energy( const or_rad_tables *t, double chi, double dt )
{
    const double a = 1.0 + 4.8 * ( 1.0 + chi ) * log( 1.0 + 1.7 * chi ) + 2.44 * chi * chi;
    return ( 1.0 / cbrt( a * a ) ) * dt * chi * chi * t->factor_classical;
}

/* RadiationMonteCarlo::operator() (RadiationMonteCarlo.cpp:62-611) without macro-photon
 * creation: the emitted energy is tallied (the branch taken when no photon species is
 * given, :545-551).  Per particle, the random draws come from its own counter-based
 * stream (id = first_id + index, step).  Returns the radiated energy sum_p w * dgamma
 * (times mass is up to the caller) and stores each particle's chi after the pass.
 * photon_chi_fn: 0 = table, else user callback (not used by the oracle). */
/* Macro-photon output of a Monte-Carlo pass (RadiationMonteCarlo.cpp:425-545): an
 * emission whose photon_gamma >= threshold, while the particle has made fewer than
 * max_emissions photons in this pass, creates `sampling` photons at the particle's
 * position with momentum photon_gamma * p / |p| (p after the recoil), weight
 * w / sampling, chi = photon_chi, tau = -1; its energy is then not added to the
 * radiated tally.  Photons are appended in particle order; count may exceed cap
 * (nothing is written past cap). */
typedef struct {
    int ndim;
    const double *pos;           /* particle positions, pos[d * n + p] */
    int sampling, max_emissions;
    double threshold;
    int64_t cap, count;
    double *ph_pos, *ph_mom, *ph_w, *ph_chi, *ph_tau; /* ph_pos[d * cap + k], ph_mom[c * cap + k] */
} or_photon_out;

static double mc_pass( const or_rad_tables *t, int64_t n, double dt, double mass, double charge,
                       double *mom, const double *weight, double *tau, double *chi_out,
                       const double *Epart, const double *Bpart, uint32_t seed, uint32_t first_id,
                       uint32_t step, int64_t *n_emissions, or_photon_out *ph );

double or_rad_monte_carlo( const or_rad_tables *t, int64_t n, double dt, double mass, double charge,
                           double *mom, const double *weight, double *tau, double *chi_out,
                           const double *Epart, const double *Bpart, uint32_t seed, uint32_t first_id,
                           uint32_t step, int64_t *n_emissions )
{
    return mc_pass( t, n, dt, mass, charge, mom, weight, tau, chi_out, Epart, Bpart, seed, first_id, step,
                    n_emissions, NULL );
}

double or_rad_monte_carlo_photons( const or_rad_tables *t, int ndim, int64_t n, double dt, double mass,
                                   double charge, const double *pos, double *mom, const double *weight,
                                   double *tau, double *chi_out, const double *Epart, const double *Bpart,
                                   uint32_t seed, uint32_t first_id, uint32_t step, int sampling,
                                   double threshold, int max_emissions, int64_t cap, double *ph_pos,
                                   double *ph_mom, double *ph_w, double *ph_chi, double *ph_tau,
                                   int64_t *n_photons, int64_t *n_emissions )
{
    or_photon_out ph = { ndim, pos, sampling, max_emissions, threshold, cap, 0, ph_pos, ph_mom, ph_w, ph_chi, ph_tau };
    const double r = mc_pass( t, n, dt, mass, charge, mom, weight, tau, chi_out, Epart, Bpart, seed, first_id, step,
                              n_emissions, &ph );
    if( n_photons ) *n_photons = ph.count;
    return r;
}

static double mc_pass( const or_rad_tables *t, int64_t n, double dt, double mass, double charge,
                       double *mom, const double *weight, double *tau, double *chi_out,
                       const double *Epart, const double *Bpart, uint32_t seed, uint32_t first_id,
                       uint32_t step, int64_t *n_emissions, or_photon_out *ph )
{
    const double oom = 1.0 / mass;
    const double qm2 = charge * oom * oom;
    const double eps_tau = 1e-100;
    const int max_it = 100;
    double radiated = 0.0;
    int64_t nem = 0;
    for( int64_t p = 0; p < n; p++ ) {
        double px = mom[p], py = mom[n + p], pz = mom[2 * n + p];
        const double Ex = Epart[p], Ey = Epart[n + p], Ez = Epart[2 * n + p];
        const double Bx = Bpart[p], By = Bpart[n + p], Bz = Bpart[2 * n + p];
        uint32_t rs = or_rng_init( seed, first_id + ( uint32_t )p, step );
        double local_time = 0.0, emission_time = 0.0;
        int it = 0, i_photon = 0;
        while( local_time < dt && it < max_it ) {
            const double g = sqrt( 1.0 + px * px + py * py + pz * pz );
            if( g < 1.1 ) break;
            const double chi = particle_chi( qm2, px, py, pz, g, Ex, Ey, Ez, Bx, By, Bz, t->inv_norm_E_schwinger );
            if( chi > t->min_chi_discontinuous && tau[p] <= eps_tau ) {
                while( tau[p] <= eps_tau ) tau[p] = -log( 1.0 - rng_uniform( &rs ) );
            }
            if( tau[p] > eps_tau ) {
                const double rate = or_rad_yield( t, chi, g );
                emission_time = fmin( tau[p] / rate, dt - local_time );
                tau[p] -= rate * emission_time;
                if( tau[p] <= eps_tau ) {
                    const double u = rng_uniform( &rs );
                    const double pchi = or_rad_photon_chi( t, chi, u );
                    const double pg = pchi / chi * ( g - 1.0 );
                    const double f = pg / sqrt( g * g - 1.0 );
                    px -= px * f;
                    py -= py * f;
                    pz -= pz * f;
                    if( ph && pg >= ph->threshold && i_photon < ph->max_emissions ) {
                        const double inv = 1.0 / sqrt( px * px + py * py + pz * pz );
                        for( int k = 0; k < ph->sampling; k++ ) {
                            const int64_t o = ph->count++;
                            if( o >= ph->cap ) continue;
                            for( int d = 0; d < ph->ndim; d++ ) ph->ph_pos[d * ph->cap + o] = ph->pos[d * n + p];
                            ph->ph_mom[o] = pg * px * inv;
                            ph->ph_mom[ph->cap + o] = pg * py * inv;
                            ph->ph_mom[2 * ph->cap + o] = pg * pz * inv;
                            ph->ph_w[o] = weight[p] * ( 1.0 / ph->sampling );
                            ph->ph_chi[o] = pchi;
                            ph->ph_tau[o] = -1.0;
                        }
                        i_photon++;
                    } else {
                        const double gn = sqrt( 1.0 + px * px + py * py + pz * pz );
                        radiated += weight[p] * ( g - gn );
                    }
                    nem++;
                    tau[p] = -1.0;
                }
                it++;
                local_time += emission_time;
            } else if( chi <= t->min_chi_discontinuous && tau[p] <= eps_tau && chi > t->min_chi_continuous ) {
                emission_time = dt - local_time;
                const double e = ridgers_energy( t, chi, emission_time );
                const double tmp = e * g / ( g * g - 1.0 );
                px -= tmp * px;
                py -= tmp * py;
                pz -= tmp * pz;
                radiated += weight[p] * ( g - sqrt( 1.0 + px * px + py * py + pz * pz ) );
                local_time = dt;
            } else {
                local_time = dt;
            }
        }
        mom[p] = px;
        mom[n + p] = py;
        mom[2 * n + p] = pz;
        if( chi_out ) { /* chi of the final momentum (RadiationMonteCarlo.cpp:642-655) */
            const double gf = sqrt( 1.0 + px * px + py * py + pz * pz );
            chi_out[p] = particle_chi( qm2, px, py, pz, gf, Ex, Ey, Ez, Bx, By, Bz, t->inv_norm_E_schwinger );
        }
    }
    if( n_emissions ) *n_emissions = nem;
    return radiated;
}

/* Batch forms for the Python harness. */
void or_rad_yield_n( const or_rad_tables *t, int64_t n, const double *chi, const double *gamma, double *out )
{
    for( int64_t i = 0; i < n; i++ ) out[i] = or_rad_yield( t, chi[i], gamma[i] );
}

void or_rad_photon_chi_n( const or_rad_tables *t, int64_t n, const double *chi, const double *xi, double *out )
{
    for( int64_t i = 0; i < n; i++ ) out[i] = or_rad_photon_chi( t, chi[i], xi[i] );
}

/* Rectilinear photon push (PusherPhoton::operator(), src/Pusher/PusherPhoton.cpp:30-85):
 * invgf = 1 / |p|, x += dt p invgf. */
void or_push_photons( int ndim, int64_t n, double dt, double *pos, const double *mom, double *invgf )
{
    for( int64_t p = 0; p < n; p++ ) {
        const double px = mom[p], py = mom[n + p], pz = mom[2 * n + p];
        const double inv = 1.0 / sqrt( px * px + py * py + pz * pz );
        if( invgf ) invgf[p] = inv;
        const double m[3] = { px, py, pz };
        for( int d = 0; d < ndim; d++ ) pos[d * n + p] += dt * m[d] * inv;
    }
}
