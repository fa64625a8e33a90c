// Test infrastructure: drives the reference's own compiled operators.
//
// oracle/build_ref.sh compiles a handful of the reference's operator sources
// (Interpolator{2D,3D}2Order, Pusher{Boris,Vay,HigueraCary},
// Projector{2D,3D}2Order, MA_Solver{2D,3D}_norm, MF_Solver{2D,3D}_Yee,
// RadiationTables, RadiationMonteCarlo) straight from the reference tree and links them with this
// file into oracle/_ref/libsmilei_ref_ops.so.  The extern "C" entry points
// below build the minimum reference objects those operators read (Params,
// Patch, Species, ElectroMagn, SmileiMPI), call the operator exactly the way
// Species::dynamics and VectorPatch::solveMaxwell do, and copy the results out.
//
// The big reference classes (Params, Patch, Species, ElectroMagn, SmileiMPI)
// have constructors that run the whole namelist machinery.  The operators
// only read a few of their members, so each is built in zero-filled storage
// and only those members are constructed in place.  This is a test harness
// and never part of the product: only the tests and the golden-fixture script
// load this library.

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <iomanip>
#include <iostream>
#include <map>
#include <memory>
#include <new>
#include <sstream>
#include <string>
#include <vector>
#include <mpi.h>
#include <hdf5.h>
#include <omp.h>
#include <Python.h>

// A few members the operators read (patch start index, table factors) are
// protected or private in the reference headers; the harness sets them
// directly.
#define private public
#define protected public
#include "Params.h"
#include "Patch.h"
#include "Species.h"
#include "SmileiMPI.h"
#include "ElectroMagn.h"
#include "Field2D.h"
#include "Field3D.h"
#include "Particles.h"
#include "Interpolator2D2Order.h"
#include "Interpolator3D2Order.h"
#include "PusherBoris.h"
#include "PusherVay.h"
#include "PusherHigueraCary.h"
#include "Projector2D2Order.h"
#include "Projector3D2Order.h"
#include "MA_Solver2D_norm.h"
#include "MA_Solver3D_norm.h"
#include "MF_Solver2D_Yee.h"
#include "MF_Solver3D_Yee.h"
#include "RadiationTables.h"
#include "RadiationTablesDefault.h"
#include "RadiationMonteCarlo.h"
#include "Random.h"
#include "ElectroMagnBC2D_SM.h"
#include "Laser.h"
#include "Profile.h"
#include "Function.h"
#undef private
#undef protected

namespace {

template <class T>
T *zeroed()
{
    void *p = nullptr;
    if( posix_memalign( &p, 64, ( ( sizeof( T ) + 63 ) / 64 ) * 64 ) != 0 ) std::abort();
    std::memset( p, 0, sizeof( T ) );
    return static_cast<T *>( p );
}

struct Geometry {
    int ndim;
    unsigned n_prim[3];   // primal sizes including ghosts (patch_size + 1 + 2*oversize)
    unsigned n_dual[3];   // n_prim + 1
    unsigned patch[3];    // patch size in cells
    unsigned oversize[3];
};

Geometry make_geom( int ndim, const int *patch_cells, const int *oversize )
{
    Geometry g{};
    g.ndim = ndim;
    for( int d = 0; d < 3; d++ ) {
        g.patch[d] = d < ndim ? patch_cells[d] : 0;
        g.oversize[d] = d < ndim ? oversize[d] : 0;
        g.n_prim[d] = d < ndim ? patch_cells[d] + 1 + 2 * oversize[d] : 1;
        g.n_dual[d] = d < ndim ? g.n_prim[d] + 1 : 1;
    }
    return g;
}

Params *make_params( const Geometry &g, const double *cell_length, double dt )
{
    Params *p = zeroed<Params>();
    new( &p->cell_length ) std::vector<double>( cell_length, cell_length + g.ndim );
    new( &p->patch_size_ ) std::vector<unsigned int>( g.patch, g.patch + g.ndim );
    new( &p->oversize ) std::vector<unsigned int>( g.oversize, g.oversize + g.ndim );
    new( &p->vectorization_mode ) std::string( "off" );
    new( &p->geometry ) std::string( g.ndim == 3 ? "3Dcartesian" : "2Dcartesian" );
    p->timestep = dt;
    p->nDim_particle = g.ndim;
    p->nDim_field = g.ndim;
    double vol = 1.0;
    for( int d = 0; d < g.ndim; d++ ) vol *= cell_length[d];
    p->cell_volume = vol;
    p->is_pxr = false;
    p->is_spectral = false;
    p->cell_sorting_ = false;
    return p;
}

Patch *make_patch( int ndim, const int *domain_begin )
{
    Patch *p = zeroed<Patch>();
    new( &p->cell_starting_global_index ) std::vector<int>( domain_begin, domain_begin + ndim );
    return p;
}

Field *make_field( const Geometry &g, int dual_x, int dual_y, int dual_z, const double *src )
{
    std::vector<unsigned int> dims;
    dims.push_back( dual_x ? g.n_dual[0] : g.n_prim[0] );
    dims.push_back( dual_y ? g.n_dual[1] : g.n_prim[1] );
    if( g.ndim == 3 ) dims.push_back( dual_z ? g.n_dual[2] : g.n_prim[2] );
    Field *f;
    if( g.ndim == 3 ) f = new Field3D( dims );
    else f = new Field2D( dims );
    std::size_t n = 1;
    for( unsigned d : dims ) n *= d;
    if( src ) std::memcpy( f->data_, src, n * sizeof( double ) );
    else std::memset( f->data_, 0, n * sizeof( double ) );
    return f;
}

std::size_t field_size( Field *f )
{
    std::size_t n = 1;
    for( unsigned d : f->dims_ ) n *= d;
    return n;
}

// Yee staggering of each component: (dual in x, dual in y, dual in z).
// Ex(d,p,p) Ey(p,d,p) Ez(p,p,d) Bx(p,d,d) By(d,p,d) Bz(d,d,p); J like E; rho primal.
const int STAG[9][3] = { {1,0,0}, {0,1,0}, {0,0,1}, {0,1,1}, {1,0,1}, {1,1,0}, {1,0,0}, {0,1,0}, {0,0,1} };

ElectroMagn *make_em( const Geometry &g, double *const *arr /* Ex Ey Ez Bx By Bz Jx Jy Jz rho Bxm Bym Bzm */ )
{
    ElectroMagn *em = zeroed<ElectroMagn>();
    new( &em->dimPrim ) std::vector<unsigned int>( g.n_prim, g.n_prim + g.ndim );
    new( &em->dimDual ) std::vector<unsigned int>( g.n_dual, g.n_dual + g.ndim );
    new( &em->Jx_s ) std::vector<Field *>( 1, nullptr );
    new( &em->Jy_s ) std::vector<Field *>( 1, nullptr );
    new( &em->Jz_s ) std::vector<Field *>( 1, nullptr );
    new( &em->rho_s ) std::vector<Field *>( 1, nullptr );
    auto st = [&]( int c, int d ) { return ( g.ndim == 2 && d == 2 ) ? 0 : STAG[c][d]; };
    em->Ex_ = make_field( g, st( 0, 0 ), st( 0, 1 ), st( 0, 2 ), arr[0] );
    em->Ey_ = make_field( g, st( 1, 0 ), st( 1, 1 ), st( 1, 2 ), arr[1] );
    em->Ez_ = make_field( g, st( 2, 0 ), st( 2, 1 ), st( 2, 2 ), arr[2] );
    em->Bx_ = make_field( g, st( 3, 0 ), st( 3, 1 ), st( 3, 2 ), arr[3] );
    em->By_ = make_field( g, st( 4, 0 ), st( 4, 1 ), st( 4, 2 ), arr[4] );
    em->Bz_ = make_field( g, st( 5, 0 ), st( 5, 1 ), st( 5, 2 ), arr[5] );
    em->Jx_ = make_field( g, st( 6, 0 ), st( 6, 1 ), st( 6, 2 ), arr[6] );
    em->Jy_ = make_field( g, st( 7, 0 ), st( 7, 1 ), st( 7, 2 ), arr[7] );
    em->Jz_ = make_field( g, st( 8, 0 ), st( 8, 1 ), st( 8, 2 ), arr[8] );
    em->rho_ = make_field( g, 0, 0, 0, arr[9] );
    em->Bx_m = make_field( g, st( 3, 0 ), st( 3, 1 ), st( 3, 2 ), arr[10] );
    em->By_m = make_field( g, st( 4, 0 ), st( 4, 1 ), st( 4, 2 ), arr[11] );
    em->Bz_m = make_field( g, st( 5, 0 ), st( 5, 1 ), st( 5, 2 ), arr[12] );
    return em;
}

void copy_back( ElectroMagn *em, double *const *arr )
{
    Field *f[13] = { em->Ex_, em->Ey_, em->Ez_, em->Bx_, em->By_, em->Bz_, em->Jx_, em->Jy_, em->Jz_, em->rho_,
                     em->Bx_m, em->By_m, em->Bz_m };
    for( int i = 0; i < 13; i++ ) {
        if( arr[i] ) std::memcpy( arr[i], f[i]->data_, field_size( f[i] ) * sizeof( double ) );
    }
}

SmileiMPI *make_smpi( int ndim, int npart )
{
    SmileiMPI *s = zeroed<SmileiMPI>();
    new( &s->dynamics_Epart ) std::vector<std::vector<double>>( 1, std::vector<double>( 3 * npart ) );
    new( &s->dynamics_Bpart ) std::vector<std::vector<double>>( 1, std::vector<double>( 3 * npart ) );
    new( &s->dynamics_invgf ) std::vector<std::vector<double>>( 1, std::vector<double>( npart ) );
    new( &s->dynamics_iold ) std::vector<std::vector<int>>( 1, std::vector<int>( ndim * npart ) );
    new( &s->dynamics_deltaold ) std::vector<std::vector<double>>( 1, std::vector<double>( ndim * npart ) );
    s->use_BTIS3 = false;
    return s;
}

void fill_particles( Particles &p, int ndim, int npart, const double *pos, const double *mom, const double *w,
                     const short *q )
{
    p.initialize( npart, ndim, false );
    for( int d = 0; d < ndim; d++ )
        for( int i = 0; i < npart; i++ ) p.Position[d][i] = pos ? pos[d * npart + i] : 0.0;
    for( int d = 0; d < 3; d++ )
        for( int i = 0; i < npart; i++ ) p.Momentum[d][i] = mom ? mom[d * npart + i] : 0.0;
    for( int i = 0; i < npart; i++ ) {
        p.Weight[i] = w ? w[i] : 1.0;
        p.Charge[i] = q ? q[i] : -1;
    }
    p.first_index.assign( 1, 0 );
    p.last_index.assign( 1, npart );
}

} // namespace

extern "C" {

// Interpolator{2D,3D}2Order::fieldsWrapper (Interpolator3D2Order.cpp:163).
// fields: Ex Ey Ez Bx_m By_m Bz_m in reference layout (x-major, last dim fastest).
int ref_interpolate( int ndim, const int *patch_cells, const int *oversize, const int *domain_begin,
                     const double *cell_length, double *const *fields, int npart, const double *pos,
                     double *Epart, double *Bpart, int *iold, double *delta )
{
    Geometry g = make_geom( ndim, patch_cells, oversize );
    Params *params = make_params( g, cell_length, 1.0 );
    Patch *patch = make_patch( ndim, domain_begin );
    double *arr[13] = { fields[0], fields[1], fields[2], nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                        fields[3], fields[4], fields[5] };
    ElectroMagn *em = make_em( g, arr );
    SmileiMPI *smpi = make_smpi( ndim, npart );
    Particles part;
    fill_particles( part, ndim, npart, pos, nullptr, nullptr, nullptr );
    Interpolator *interp;
    if( ndim == 3 ) interp = new Interpolator3D2Order( *params, patch );
    else interp = new Interpolator2D2Order( *params, patch );
    int istart = 0, iend = npart;
    interp->fieldsWrapper( em, part, smpi, &istart, &iend, 0 );
    std::memcpy( Epart, smpi->dynamics_Epart[0].data(), 3 * npart * sizeof( double ) );
    std::memcpy( Bpart, smpi->dynamics_Bpart[0].data(), 3 * npart * sizeof( double ) );
    std::memcpy( iold, smpi->dynamics_iold[0].data(), ndim * npart * sizeof( int ) );
    std::memcpy( delta, smpi->dynamics_deltaold[0].data(), ndim * npart * sizeof( double ) );
    return 0;
}

// Pusher{Boris,Vay,HigueraCary}::operator() (PusherBoris.cpp:23, PusherVay.cpp:32, PusherHigueraCary.cpp:32).
// kind: 0 boris, 1 vay, 2 higueracary.  pos/mom updated in place; invgf written.
int ref_push( int kind, int ndim, double dt, double mass, int npart, double *pos, double *mom, const short *charge,
              const double *Epart, const double *Bpart, double *invgf )
{
    int cells[3] = { 8, 8, 8 }, os[3] = { 2, 2, 2 };
    double cl[3] = { 1.0, 1.0, 1.0 };
    Geometry g = make_geom( ndim, cells, os );
    Params *params = make_params( g, cl, dt );
    Species *sp = zeroed<Species>();
    sp->mass_ = mass;
    SmileiMPI *smpi = make_smpi( ndim, npart );
    std::memcpy( smpi->dynamics_Epart[0].data(), Epart, 3 * npart * sizeof( double ) );
    std::memcpy( smpi->dynamics_Bpart[0].data(), Bpart, 3 * npart * sizeof( double ) );
    Particles part;
    fill_particles( part, ndim, npart, pos, mom, nullptr, charge );
    Pusher *push;
    if( kind == 0 ) push = new PusherBoris( *params, sp );
    else if( kind == 1 ) push = new PusherVay( *params, sp );
    else push = new PusherHigueraCary( *params, sp );
    ( *push )( part, smpi, 0, npart, 0, 0 );
    for( int d = 0; d < ndim; d++ )
        for( int i = 0; i < npart; i++ ) pos[d * npart + i] = part.Position[d][i];
    for( int d = 0; d < 3; d++ )
        for( int i = 0; i < npart; i++ ) mom[d * npart + i] = part.Momentum[d][i];
    std::memcpy( invgf, smpi->dynamics_invgf[0].data(), npart * sizeof( double ) );
    return 0;
}

// Projector{2D,3D}2Order::currentsAndDensityWrapper (Projector3D2Order.cpp:733, Projector2D2Order.cpp:498)
// and ::basic (Projector3D2Order.cpp:526).
// mode 0: currents (J only); 1: currentsAndDensity (diag step, J and rho); 2: basic rho projection.
// J: Jx Jy Jz rho, accumulated into (the caller passes the initial values).
int ref_project( int mode, int ndim, const int *patch_cells, const int *oversize, const int *domain_begin,
                 const double *cell_length, double dt, int npart, const double *pos, const double *mom,
                 const double *weight, const short *charge, const double *invgf, const int *iold,
                 const double *delta, double *const *J )
{
    Geometry g = make_geom( ndim, patch_cells, oversize );
    Params *params = make_params( g, cell_length, dt );
    Patch *patch = make_patch( ndim, domain_begin );
    double *arr[13] = { nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, J[0], J[1], J[2], J[3],
                        nullptr, nullptr, nullptr };
    ElectroMagn *em = make_em( g, arr );
    SmileiMPI *smpi = make_smpi( ndim, npart );
    if( invgf ) std::memcpy( smpi->dynamics_invgf[0].data(), invgf, npart * sizeof( double ) );
    if( iold ) std::memcpy( smpi->dynamics_iold[0].data(), iold, ndim * npart * sizeof( int ) );
    if( delta ) std::memcpy( smpi->dynamics_deltaold[0].data(), delta, ndim * npart * sizeof( double ) );
    Particles part;
    fill_particles( part, ndim, npart, pos, mom, weight, charge );
    Projector *proj;
    if( ndim == 3 ) proj = new Projector3D2Order( *params, patch );
    else proj = new Projector2D2Order( *params, patch );
    if( mode == 0 || mode == 1 ) {
        proj->currentsAndDensityWrapper( em, part, smpi, 0, npart, 0, mode == 1, false, 0 );
    } else {
        double *rho = em->rho_->data_;
        for( int i = 0; i < npart; i++ ) proj->basic( rho, part, i, 0 );
    }
    double *out[13] = { nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, J[0], J[1], J[2], J[3],
                        nullptr, nullptr, nullptr };
    copy_back( em, out );
    return 0;
}

// MA_Solver{2D,3D}_norm (which=0) and MF_Solver{2D,3D}_Yee (which=1) on one patch's arrays.
// F: Ex Ey Ez Bx By Bz Jx Jy Jz, updated in place.
int ref_maxwell( int which, int ndim, const int *patch_cells, const int *oversize, const double *cell_length,
                 double dt, double *const *F )
{
    Geometry g = make_geom( ndim, patch_cells, oversize );
    Params *params = make_params( g, cell_length, dt );
    double *arr[13] = { F[0], F[1], F[2], F[3], F[4], F[5], F[6], F[7], F[8], nullptr, nullptr, nullptr, nullptr };
    ElectroMagn *em = make_em( g, arr );
    Solver *s;
    if( which == 0 ) s = ndim == 3 ? ( Solver * )new MA_Solver3D_norm( *params ) : ( Solver * )new MA_Solver2D_norm( *params );
    else s = ndim == 3 ? ( Solver * )new MF_Solver3D_Yee( *params ) : ( Solver * )new MF_Solver2D_Yee( *params );
    ( *s )( em );
    double *out[13] = { F[0], F[1], F[2], F[3], F[4], F[5], nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr };
    copy_back( em, out );
    return 0;
}

// RadiationTables with the default tables (RadiationTables.cpp:164 setDefault branch).
static RadiationTables *g_rad = nullptr;

static RadiationTables *rad()
{
    if( !g_rad ) {
        g_rad = new RadiationTables();
        RadiationTablesDefault::setDefault( g_rad->niel_, g_rad->integfochi_, g_rad->xi_ );
    }
    return g_rad;
}

// Table geometry: sizes and axis bounds of the default integfochi and xi tables.
int ref_rad_table_info( int *integ_size, double *integ_min, double *integ_max, int *xi_dims, double *xi_min,
                        double *xi_max )
{
    RadiationTables *r = rad();
    *integ_size = r->integfochi_.size_;
    *integ_min = r->integfochi_.min_;
    *integ_max = r->integfochi_.max_;
    xi_dims[0] = r->xi_.dim_size_[0];
    xi_dims[1] = r->xi_.dim_size_[1];
    *xi_min = r->xi_.min_;
    *xi_max = r->xi_.max_;
    return 0;
}

// Copies the default table contents out (integfochi[size], xi[dim0*dim1], xi axis1 min[dim0]).
int ref_rad_table_data( double *integ, double *xi, double *xi_axis1_min )
{
    RadiationTables *r = rad();
    std::memcpy( integ, r->integfochi_.data_, r->integfochi_.size_ * sizeof( double ) );
    std::memcpy( xi, r->xi_.data_, r->xi_.dim_size_[0] * r->xi_.dim_size_[1] * sizeof( double ) );
    std::memcpy( xi_axis1_min, r->xi_.axis1_min_, r->xi_.dim_size_[0] * sizeof( double ) );
    return 0;
}

// RadiationTables::computePhotonProductionYield (RadiationTables.cpp:225), with factor_dNph_dt_ given.
int ref_rad_yield( int n, const double *chi, const double *gamma, double factor_dNph_dt, double *out )
{
    RadiationTables *r = rad();
    r->factor_dNph_dt_ = factor_dNph_dt;
    for( int i = 0; i < n; i++ ) out[i] = r->computePhotonProductionYield( chi[i], gamma[i] );
    return 0;
}

// RadiationTables::computeRandomPhotonChiWithInterpolation (RadiationTables.cpp:375).
int ref_rad_photon_chi( int n, const double *chi, const double *xi, double *out )
{
    RadiationTables *r = rad();
    for( int i = 0; i < n; i++ ) out[i] = r->computeRandomPhotonChiWithInterpolation( chi[i], xi[i] );
    return 0;
}

// RadiationMonteCarlo::operator() (RadiationMonteCarlo.cpp:62-656) with the default
// tables, as Species::dynamics calls it (Species.cpp:615): particle p alone in each call
// (istart = p, iend = p + 1) and with its own Random(seeds[p]), so that its draws are the
// xorshift32 stream started from seeds[p].  The table factors, the chi thresholds and
// 1/E_Schwinger are given (RadiationTables::initialization and the Radiation constructor
// read them from the namelist).  sampling > 0 passes a photon species with chi and tau
// (Species.cpp:615 with a radiation_photon_species); its photons, in creation order, are
// copied out up to cap (ph_pos[d * cap + k], ph_mom[c * cap + k]) and *n_photons counts
// them all.  mom[c * n + p], Epart/Bpart[c * n + p]; mom, tau and chi are updated.
int ref_monte_carlo( int ndim, int n, double dt, double mass, double charge, double factor_dNph_dt,
                     double factor_classical, double min_chi_continuous, double min_chi_discontinuous,
                     double inv_norm_E_schwinger, const double *pos, double *mom, const double *weight, double *tau,
                     double *chi, const double *Epart, const double *Bpart, const unsigned *seeds, int sampling,
                     double threshold, int max_emissions, long cap, double *ph_pos, double *ph_mom, double *ph_w,
                     double *ph_chi, double *ph_tau, long *n_photons, double *radiated )
{
    RadiationTables *r = rad();
    r->factor_dNph_dt_ = factor_dNph_dt;
    r->factor_classical_radiated_power_ = factor_classical;
    r->minimum_chi_continuous_ = min_chi_continuous;
    r->minimum_chi_discontinuous_ = min_chi_discontinuous;
    Params *params = zeroed<Params>();
    params->nDim_particle = ndim;
    params->timestep = dt;
    Species *sp = zeroed<Species>();
    sp->mass_ = mass;
    sp->radiation_photon_sampling_ = sampling > 0 ? sampling : 1;
    sp->radiation_max_emissions_ = max_emissions;
    sp->radiation_photon_gamma_threshold_ = threshold;
    Random seed0( 1u );
    RadiationMonteCarlo mc( *params, sp, &seed0 );
    // the Params constants behind E_Schwinger are not constructed in the zero-filled Params
    mc.inv_norm_E_Schwinger_ = inv_norm_E_schwinger;
    mc.norm_E_Schwinger_ = 1.0 / inv_norm_E_schwinger;

    SmileiMPI *smpi = make_smpi( ndim, n );
    std::memcpy( smpi->dynamics_Epart[0].data(), Epart, 3 * ( std::size_t )n * sizeof( double ) );
    std::memcpy( smpi->dynamics_Bpart[0].data(), Bpart, 3 * ( std::size_t )n * sizeof( double ) );
    std::vector<short> q( n, ( short )charge );
    Particles part;
    part.has_quantum_parameter = true;
    part.has_Monte_Carlo_process = true;
    fill_particles( part, ndim, n, pos, mom, weight, q.data() );
    for( int p = 0; p < n; p++ ) {
        part.Tau[p] = tau[p];
        part.Chi[p] = 0.0;
    }
    Particles photons;
    photons.has_quantum_parameter = true;
    photons.has_Monte_Carlo_process = true;
    photons.initialize( 0, ndim, false );

    double total = 0.0;
    for( int p = 0; p < n; p++ ) {
        Random rnd( seeds[p] );
        mc.rand_ = &rnd;
        mc( part, sampling > 0 ? &photons : nullptr, smpi, *r, total, p, p + 1, 0, 0, 0 );
    }
    mc.rand_ = &seed0;
    *radiated = total;
    for( int c = 0; c < 3; c++ )
        for( int p = 0; p < n; p++ ) mom[c * n + p] = part.Momentum[c][p];
    for( int p = 0; p < n; p++ ) {
        tau[p] = part.Tau[p];
        chi[p] = part.Chi[p];
    }
    const long np = sampling > 0 ? ( long )photons.size() : 0;
    *n_photons = np;
    for( long k = 0; k < np && k < cap; k++ ) {
        for( int d = 0; d < ndim; d++ ) ph_pos[d * cap + k] = photons.Position[d][k];
        for( int c = 0; c < 3; c++ ) ph_mom[c * cap + k] = photons.Momentum[c][k];
        ph_w[k] = photons.Weight[k];
        ph_chi[k] = photons.Chi[k];
        ph_tau[k] = photons.Tau[k];
    }
    return 0;
}

// One side of the reference's 2D Silver-Mueller condition
// (ElectroMagnBC2D_SM::apply, ElectroMagnBC2D_SM.cpp:118-265) on a single patch.
// Tangent ends are boundaries when tmin/tmax are set.  With lt != NULL a separable
// laser (LaserProfileSeparable, Laser.cpp:287-302,453-460) is attached: its time
// profile is the compiled tgaussian (Function_TimeGaussian, Function.cpp:528-535;
// lt = {start, end, invsigma, center, order}), its chirp the constant 1, and its
// space envelope and phase are given per point (sp1/ph1 on the primal points along
// the side, sp2/ph2 on the dual points), with delays d1, d2 and frequency omega.
int ref_sm_apply_2d( int side, const int *patch_cells, const int *oversize, const double *cell_length, double dt,
                     double *const *F, int tmin, int tmax, const double *lt, double omega, const double *sp1,
                     const double *ph1, double d1, const double *sp2, const double *ph2, double d2, double time_dual )
{
    Geometry g = make_geom( 2, patch_cells, oversize );
    Params *params = make_params( g, cell_length, dt );
    static const double kdef[4][2] = { { 1.0, 0.0 }, { -1.0, 0.0 }, { 0.0, 1.0 }, { 0.0, -1.0 } };
    new( &params->EM_BCs_k ) std::vector<std::vector<double>>();
    for( int k = 0; k < 4; k++ ) params->EM_BCs_k.push_back( std::vector<double>( kdef[k], kdef[k] + 2 ) );
    const int begin[2] = { -oversize[0], -oversize[1] };
    Patch *patch = make_patch( 2, begin );
    new( &patch->size_ ) std::vector<unsigned int>( g.patch, g.patch + 2 );
    new( &patch->oversize ) std::vector<unsigned int>( g.oversize, g.oversize + 2 );
    new( &patch->min_local_ ) std::vector<double>( 2, 0.0 );
    new( &patch->neighbor_ ) std::vector<std::vector<int>>( 2, std::vector<int>( 2, 0 ) );
    const int ax = side / 2, tan = ax == 0 ? 1 : 0;
    patch->neighbor_[ax][0] = patch->neighbor_[ax][1] = MPI_PROC_NULL;
    if( tmin ) patch->neighbor_[tan][0] = MPI_PROC_NULL;
    if( tmax ) patch->neighbor_[tan][1] = MPI_PROC_NULL;
    double *arr[13] = { F[0], F[1], F[2], F[3], F[4], F[5], nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr };
    ElectroMagn *em = make_em( g, arr );
    new( &em->oversize ) std::vector<unsigned int>( g.oversize, g.oversize + 2 );
    ElectroMagnBC2D_SM *bc = new ElectroMagnBC2D_SM( *params, patch, ( unsigned int )side );
    if( lt ) {
        Function_TimeGaussian *tmpl = zeroed<Function_TimeGaussian>();
        tmpl->start = lt[0];
        tmpl->end = lt[1];
        tmpl->invsigma = lt[2];
        tmpl->center = lt[3];
        tmpl->order = lt[4];
        Function_TimeConstant *ctmpl = zeroed<Function_TimeConstant>();
        ctmpl->start = -1e300;
        Profile *tprof[2], *cprof[2];
        for( int k = 0; k < 2; k++ ) {
            tprof[k] = zeroed<Profile>();
            tprof[k]->function_ = new Function_TimeGaussian( tmpl );
            cprof[k] = zeroed<Profile>();
            cprof[k]->function_ = new Function_TimeConstant( ctmpl );
        }
        Laser *laser = zeroed<Laser>();
        new( &laser->profiles ) std::vector<LaserProfile *>();
        const unsigned n1p = g.n_prim[tan], n1d = g.n_dual[tan];
        for( int k = 0; k < 2; k++ ) {
            LaserProfileSeparable *lp = new LaserProfileSeparable( omega, cprof[k], tprof[k], nullptr, nullptr,
                                                                   k == 0 ? d1 : d2, k == 0, ( unsigned int )ax );
            const unsigned n = k == 0 ? n1p : n1d;
            std::vector<unsigned int> dims = { n, 1 };
            lp->space_envelope = new Field2D( dims );
            lp->phase = new Field2D( dims );
            for( unsigned j = 0; j < n; j++ ) {
                ( *lp->space_envelope )( j, 0 ) = ( k == 0 ? sp1 : sp2 )[j];
                ( *lp->phase )( j, 0 ) = ( k == 0 ? ph1 : ph2 )[j];
            }
            laser->profiles.push_back( lp );
        }
        bc->vecLaser.push_back( laser );
    }
    bc->apply( em, time_dual, patch );
    double *out[13] = { F[0], F[1], F[2], F[3], F[4], F[5], nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr };
    copy_back( em, out );
    return 0;
}

} // extern "C"
