/* smilei_gb300.h -- C ABI of libsmileigb300.so, the GB300 (sm_103a) PIC-step hot path.
 *
 * Every entry point is extern "C", takes plain pointers and sizes, runs on the
 * caller's CUDA stream (NULL = legacy default stream), returns an int status
 * (SG_OK = 0, negative on error) and never exits the process.  The text of
 * the last error of the calling thread is returned by sg_last_error().
 *
 * Data layout is the reference's (Smilei):
 *   - fields: one array per component, x-major with the last dimension
 *     fastest, ghost cells included; a primal dimension has
 *     n_cells + 1 + 2*oversize points and a dual one has one more
 *     (src/ElectroMagn/ElectroMagn3D.cpp:115-123, src/Params/Params.cpp:1202-1207).
 *     Staggering Ex(d,p,p) Ey(p,d,p) Ez(p,p,d) Bx(p,d,d) By(d,p,d) Bz(d,d,p),
 *     J like E, rho primal; in 2D the third index is dropped.
 *   - particles: structure of arrays, absolute positions pos[d*n + i],
 *     momenta mom[d*n + i], weight[i], charge[i] (short)
 *     (src/Particles/Particles.h:48, property order Particles.cpp:71-98).
 *   - interpolator -> pusher -> projector scratch Epart[3n], Bpart[3n],
 *     invgf[n], iold[ndim*n] (int), deltaold[ndim*n]
 *     (src/SmileiMPI/SmileiMPI.h:213-221).
 * Pointers given to the operator entry points are device pointers.
 */
#ifndef SMILEI_GB300_H
#define SMILEI_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SG_OK 0
#define SG_ERR_ARG (-1)        /* invalid argument */
#define SG_ERR_CUDA (-2)       /* a CUDA runtime call failed */
#define SG_ERR_BOUNDS (-3)     /* a particle left the region its kernel can reach (device check) */
#define SG_ERR_OVERFLOW (-4)   /* a capacity was exceeded and could not be grown */
#define SG_ERR_STATE (-5)      /* call not valid in the object's current state */
#define SG_ERR_NOMEM (-6)      /* device allocation failed */

typedef void *sg_stream_t; /* a cudaStream_t */

/* Geometry of one patch's field arrays.
 * n_prim[d]       primal extent with ghosts (patch_size[d] + 1 + 2*oversize[d])
 * domain_begin[d] global index of local point 0 (patch start - oversize),
 *                 as src/Interpolator/Interpolator3D.cpp:14-16 and
 *                 src/Projector/Projector3D2Order.cpp:29-31 compute it. */
typedef struct sg_grid_geom {
    int ndim;
    int n_prim[3];
    int domain_begin[3];
    double cell_length[3];
} sg_grid_geom;

const char *sg_last_error( void );
int sg_version( void );

/* ---- operator entry points (FP64, the reference's arrays on the device) ---- */

/* Order-2 gather of E and B_m at the particles.
 * Replaces Interpolator3D2Order::fieldsWrapper / Interpolator2D2Order::fieldsWrapper
 * (src/Interpolator/Interpolator.h:23, Interpolator3D2Order.cpp:163,
 * Interpolator2D2Order.cpp:158).  fields = {Ex, Ey, Ez, Bx_m, By_m, Bz_m}. */
int sg_interpolate_fields( const sg_grid_geom *geom, const double *const *fields, int64_t npart,
                           const double *pos, double *Epart, double *Bpart, int *iold, double *deltaold,
                           sg_stream_t stream );

/* Particle push; kind 0 = Boris, 1 = Vay, 2 = Higuera-Cary.
 * Replaces Pusher::operator() (src/Pusher/Pusher.h:22; PusherBoris.cpp:23,
 * PusherVay.cpp:32, PusherHigueraCary.cpp:32).  pos/mom updated in place. */
int sg_push_particles( int kind, int ndim, double dt, double mass, int64_t npart, double *pos, double *mom,
                       const short *charge, const double *Epart, const double *Bpart, double *invgf,
                       sg_stream_t stream );

/* Charge-conserving (Esirkepov) deposit, accumulated into J.
 * mode 0: currents; 1: currents and rho (diagnostic step); 2: rho only from the
 * current positions (Projector3D2Order::basic, used at initialisation).
 * Replaces Projector::currentsAndDensityWrapper (src/Projector/Projector.h:44;
 * Projector3D2Order.cpp:733, Projector2D2Order.cpp:498) and the reference's own
 * device entry point currentDeposition3DOnDevice
 * (src/Projector/Projector3D2OrderGPUKernel.cpp:40).
 * J = {Jx, Jy, Jz, rho}; unused entries may be NULL. */
int sg_project_currents( int mode, const sg_grid_geom *geom, double dt, int64_t npart, const double *pos,
                         const double *mom, const double *weight, const short *charge, const double *invgf,
                         const int *iold, const double *deltaold, double *const *J, sg_stream_t stream );

/* Yee solver on one patch.  F = {Ex, Ey, Ez, Bx, By, Bz, Jx, Jy, Jz}.
 * Ampere replaces MA_Solver3D_norm/MA_Solver2D_norm::operator()
 * (src/ElectroMagnSolver/MA_Solver3D_norm.cpp:18), all points.
 * Faraday replaces MF_Solver3D_Yee/MF_Solver2D_Yee::operator()
 * (src/ElectroMagnSolver/MF_Solver3D_Yee.cpp:18), interior points. */
int sg_maxwell_ampere( const sg_grid_geom *geom, double dt, double *const *F, sg_stream_t stream );
int sg_maxwell_faraday( const sg_grid_geom *geom, double dt, double *const *F, sg_stream_t stream );

/* B_m <- B and B_m <- (B + B_m)/2 on all points.  B = {Bx, By, Bz}, Bm likewise.
 * Replace ElectroMagn3D::saveMagneticFields / centerMagneticFields
 * (src/ElectroMagn/ElectroMagn3D.cpp:1048, :1191). */
int sg_save_magnetic_fields( const sg_grid_geom *geom, double *const *B, double *const *Bm, sg_stream_t stream );
int sg_center_magnetic_fields( const sg_grid_geom *geom, double *const *B, double *const *Bm, sg_stream_t stream );

/* Per-cell particle sort.  key = sum_d (round(x_d/dx_d) - round(xmin_d/dx_d)) * stride_d
 * over the (patch_size+1)^ndim node lattice (src/Species/SpeciesV.cpp:766-857);
 * counts -> prefix sum -> first_index/last_index (SpeciesV.cpp:645-652); then every
 * double property (pos[ndim], mom[3], weight, and any extra arrays) and the charge are
 * permuted so each cell's particles are contiguous (stable: original order kept inside
 * a cell).  Replaces Species::sortParticles (src/Species/Species.cpp:1046) for
 * particles that stay in the patch.  A particle whose key falls outside the lattice
 * is an error (SG_ERR_BOUNDS).
 * dprops: n_dprops device arrays of npart doubles; scratch is allocated internally. */
int sg_sort_particles( int ndim, const int *patch_size, const double *xmin, const double *cell_length,
                       int64_t npart, double *const *dprops, int n_dprops, short *charge, int *first_index,
                       int *last_index, int *cell_keys, sg_stream_t stream );

/* The same per-cell sort with no device allocation.  It has no counterpart in the
 * reference.  It is for callers that cannot call cudaMalloc: a host code that takes
 * the GPU's memory into its own pool at start-up leaves nothing for a library to
 * allocate later, and one that gives each library a fixed device-memory budget
 * cannot let a call grow it.  Its scratch is a fixed array in the library's device
 * image (SG_SORT_NOALLOC_SCRATCH_BYTES, held on every GPU that loads the library until
 * the process exits), so it accepts at most SG_SORT_NOALLOC_MAX_PARTICLES particles and
 * SG_SORT_NOALLOC_MAX_CELLS cells ((patch_size+1)^ndim) and returns SG_ERR_ARG beyond
 * them, before any GPU work.  The first call on a device looks the array's device
 * address up (with that device current); make that first call before any stream
 * capture.  The call waits for its stream before it returns (it reads the status
 * word).  All calls share the one array, which keeps the last call's contents: calls
 * whose GPU work overlaps (other streams, other threads) race and must be serialised
 * by the caller.  Arguments and results as sg_sort_particles. */
#define SG_SORT_NOALLOC_MAX_PARTICLES 262144
#define SG_SORT_NOALLOC_MAX_CELLS 32768
#define SG_SORT_NOALLOC_SCRATCH_BYTES ( 5 * 1024 * 1024 )
int sg_sort_particles_noalloc( int ndim, const int *patch_size, const double *xmin, const double *cell_length,
                               int64_t npart, double *const *dprops, int n_dprops, short *charge, int *first_index,
                               int *last_index, int *cell_keys, sg_stream_t stream );

/* ---- simulation object: the whole timestep resident on one GPU ---- */

/* Form of the particle/field arithmetic. */
#define SG_FORM_FP64 0  /* absolute FP64 positions, FP64 fields and currents (the reference's) */
#define SG_FORM_MIXED 1 /* int cell index + FP32 in-cell offset, FP32 momenta/fields/currents */

typedef struct sg_sim_config {
    int ndim;              /* 2 or 3 */
    int form;              /* SG_FORM_FP64 or SG_FORM_MIXED */
    int n_cells[3];        /* global cells per dimension, at least 8; the mixed form packs a
                              particle's node into one 32-bit key (3D x:11 y:10 z:10 bits, 2D
                              16:16), so it takes at most 2048 x 1024 x 1024 nodes in 3D and
                              65536 x 65536 in 2D (an open axis has one node more than cells);
                              sg_sim_create refuses larger grids in that form */
    double cell_length[3];
    double dt;
    int tile[3];           /* cells per tile (bin) per dimension; 0 = choose automatically */
    double capacity_slack; /* extra room per tile, as a fraction of its count (e.g. 0.25) */
    int use_graph;         /* capture each timestep as a CUDA graph */
    int bc[3];             /* per dimension: SG_BC_PERIODIC, or SG_BC_OPEN (2D only): Silver-Mueller
                              field boundaries (ElectroMagnBC2D_SM) on both sides and particles removed
                              when they leave (remove_particle_inf/_sup) */
} sg_sim_config;

#define SG_BC_PERIODIC 0
#define SG_BC_OPEN 1

typedef struct sg_sim sg_sim;
typedef struct sg_rad_tables sg_rad_tables; /* radiation tables (below) */
typedef struct sg_mlp sg_mlp;               /* learned inverse CDF (below) */

int sg_sim_create( const sg_sim_config *cfg, sg_sim **out );
int sg_sim_destroy( sg_sim *sim );

/* How the particle kernel's CTAs get their tiles.  on = 0 (default): one CTA per tile,
 * handed out by the hardware block scheduler.  on = 1: a persistent grid (as many CTAs
 * as fit on the GPU at once) whose CTAs take tiles from a device counter until none is
 * left, densest tile first (order recomputed at every re-layout).  The reference hands
 * patches to OpenMP threads with schedule(runtime) (src/Patch/VectorPatch.cpp:4777);
 * this is the GPU's version of that work queue.  The results are the same either way.
 * No reference counterpart as an entry point. */
int sg_sim_set_tile_queue( sg_sim *sim, int on );

/* How the particle kernel stages its tile of E and B_m in shared memory (3D mixed form
 * with 4x4x4 tiles, periodic).  on = 1 (the default for such a simulation, set by
 * sg_sim_create): one thread issues a tensor-memory-accelerator copy
 * (cp.async.bulk.tensor, completion on an mbarrier) per component; the tensor maps need
 * rows of a multiple of 16 bytes, so the field kernels also write E and B_m into padded
 * arrays (six more field arrays of device memory; a copy pass refreshes them after E or
 * B_m change outside a step).  on = 0: every thread copies words
 * with cp.async; no padded arrays are written.  The results are the same either way.
 * Any other simulation refuses on = 1.  No reference counterpart (the reference's
 * gather reads the field arrays directly, Interpolator3D2Order.cpp:225-245). */
int sg_sim_set_tma_staging( sg_sim *sim, int on );

/* Adds a species from host arrays (absolute FP64 positions pos[ndim*n],
 * momenta mom[3*n], weights[n]); pusher: 0 Boris, 1 Vay, 2 Higuera-Cary.
 * Returns the species index in *index. */
int sg_sim_add_species( sg_sim *sim, double mass, double charge, int pusher, int64_t npart, const double *pos,
                        const double *mom, const double *weight, int *index );

/* Same, from device arrays (same layout), without host copies.  The call first waits
 * for all work on the device, so arrays still being written on any stream are complete
 * before they are read. */
int sg_sim_add_species_device( sg_sim *sim, double mass, double charge, int pusher, int64_t npart,
                               const double *pos, const double *mom, const double *weight, int *index );

/* Field access, reference layout with ghosts, FP64, host buffers.
 * comp: 0..2 Ex Ey Ez, 3..5 Bx By Bz, 6..8 Bx_m By_m Bz_m, 9..11 Jx Jy Jz. */
int sg_sim_set_field( sg_sim *sim, int comp, const double *host );
int sg_sim_get_field( sg_sim *sim, int comp, double *host );
int sg_sim_field_shape( sg_sim *sim, int comp, int *shape3 );

/* Runs nsteps full timesteps (gather, push, deposit, bin sort, J ghost fold,
 * Ampere, Faraday, B centring) on the simulation's stream.  With graphs on
 * (use_graph), steps go in batches of up to 8 as one graph: each step sits behind a
 * conditional node that a one-thread gate kernel arms from the previous step's device
 * flags, so a spill or an error stops the batch on the device and the host waits once
 * per batch; the host then re-lays out a spilled species and goes on.  Steps at which
 * the moving window shifts run one by one.  After a batch, sg_sim_last_timing reports
 * -1 for the stage times (a batch records no stage events). */
int sg_sim_step( sg_sim *sim, int nsteps );

/* Batched graphs launched so far and the steps they made (sg_sim_step); *unsupported
 * is 1 when the runtime refused a batched graph and steps run one by one. */
int sg_sim_batch_stats( sg_sim *sim, int64_t *batches, int64_t *steps, int *unsupported );

/* Synchronises and copies a species back as absolute FP64 positions, momenta and
 * weights (sorted by tile; the order is not the input order).  *npart receives the
 * count; the arrays must hold at least that many particles. */
int sg_sim_species_count( sg_sim *sim, int species, int64_t *npart );
int sg_sim_get_species( sg_sim *sim, int species, double *pos, double *mom, double *weight );

/* Energy diagnostics (FP64 device reductions): kinetic energy per species summed,
 * sum_p w m (gamma - 1), and field energy 0.5 * sum (E^2 + B_m^2) * V_cell over the
 * interior points (src/Diagnostic/DiagnosticScalar.cpp:174-277). */
int sg_sim_energy( sg_sim *sim, double *ukin, double *uelm );

/* Per-species and per-field scalars of DiagnosticScalar::compute
 * (src/Diagnostic/DiagnosticScalar.cpp:470-700), FP64 device reductions.
 * sg_sim_species_scalars: out[4] = {Dens = sum w, Ntot, Zavg numerator q sum w,
 * Ukin = m sum w (gamma - 1)}.  sg_sim_field_energies: out[6] = 0.5 V_cell sum F^2
 * for Ex, Ey, Ez, Bx_m, By_m, Bz_m over the N physical points per dimension. */
int sg_sim_species_scalars( sg_sim *sim, int species, double *out );
int sg_sim_field_energies( sg_sim *sim, double *out );

/* Charge density of all species at the current positions, FP64, reference layout
 * (primal, ghosts, periodic copies folded): the basic() projection of
 * src/Projector/Projector3D2Order.cpp:526-618 summed over species. */
int sg_sim_get_rho( sg_sim *sim, double *host );

/* Initial electrostatic field: FP64 conjugate gradient for Laplacian(phi) = -rho on
 * the periodic lattice, rho of all species with its mean removed (a uniform
 * neutralising background), then E_d = (phi(i-1) - phi(i)) / dx_d with each
 * component's mean removed.  Follows VectorPatch::solvePoisson
 * (src/Patch/VectorPatch.cpp:1523-1620) and ElectroMagn3D::initPoisson, compute_Ap,
 * update_pand_r, update_p, initE (src/ElectroMagn/ElectroMagn3D.cpp:255-560);
 * stops when r.r / n_nodes <= max_error (the reference's poisson_max_error, 1e-14)
 * or after max_iter iterations (poisson_max_iteration, 50000).  Overwrites E. */
int sg_sim_solve_poisson( sg_sim *sim, double max_error, int max_iter, int *iterations, double *ctrl );

/* Charge-conservation residual max|div E - (rho - <rho>)| / max|rho - <rho>| over the
 * physical nodes, with rho deposited in FP64 from the current particles.
 * rho_max (optional) receives max|rho - <rho>|. */
int sg_sim_charge_residual( sg_sim *sim, double *residual, double *rho_max );

/* Raw particle state of a species (the library's own SoA layout, tile segments
 * included): its size, and a copy of the current buffer to (to_device = 0) or
 * from (to_device = 1) a host buffer of that size, on the simulation's stream
 * (asynchronous with pinned host memory).  A copy taken and restored unchanged
 * leaves the simulation as it was; this is how a caller that keeps particles in
 * host memory drives the resident step. */
int sg_sim_state_bytes( sg_sim *sim, int species, size_t *bytes );
int sg_sim_copy_state( sg_sim *sim, int species, void *host, int to_device );

/* The same state packed: an int64 particle count, the per-tile counts, then every
 * tile's particles back to back, plane by plane (no segment slack or holes, about 20 %
 * fewer bytes than the raw state).  pack copies it device -> host (asynchronous with
 * pinned memory); unpack copies it host -> device into the current layout, where every
 * tile's count must fit its segment (it synchronises to check that; a species'
 * optical depths stay on the device).  Restoring what was packed leaves the simulation
 * as it was. */
int sg_sim_packed_bytes( sg_sim *sim, int species, size_t *bytes );
int sg_sim_pack_state( sg_sim *sim, int species, void *host );
int sg_sim_unpack_state( sg_sim *sim, int species, const void *host );

/* One step of a species whose particles live in host memory between steps (the
 * reference's Particles vectors on the host, src/Particles/Particles.h:48): reads the
 * packed state from host_in, steps the whole simulation, and writes the new packed
 * state to host_out (host_out may equal host_in; it needs packed_bytes() bytes, and
 * particles removed at open boundaries only shrink it; it must not overlap host_in
 * unless it is host_in).  The copy in runs in `chunks` (1..64) tile ranges of about
 * equal particle counts on a second stream, and each range is stepped as soon as it is
 * in.  On a grid periodic in every dimension with at least three x-slabs of tiles,
 * each range is also packed once its neighbours have stepped and copied out on a third
 * stream, so both directions of the host link and the kernel overlap; otherwise, or
 * after a spill, the state is packed after the step.  Same result as unpack_state,
 * step(1), pack_state (up to the order of floating-point atomics in the current
 * deposit).  Not for a radiating species or a step in which the window moves.  Waits
 * for the simulation's stream first and returns after host_out is written. */
int sg_sim_step_host( sg_sim *sim, int species, const void *host_in, void *host_out, int chunks );

/* The tile ranges sg_sim_step_host uses, in processing order, for a grid of
 * ntiles[0..ndim) tiles (x-major) holding counts[t] particles per tile: range j is
 * tiles [ta[j], tb[j]).  pack_after[j] is the range after whose particle step range j's
 * output is final (-1 for all when the step does not pack while stepping: a grid not
 * periodic in every dimension, or fewer than three x-slabs of tiles).  Arrays of
 * chunks + 1 entries; host only. */
int sg_stream_ranges( int ndim, const int *ntiles, int periodic, const int *counts, int chunks, int *ta, int *tb,
                      int *pack_after, int *nranges );

/* Stage times of the last sg_sim_step_host that packed while stepping, in ms from its
 * start (-1 where not measured): [0] copy in done, [1] particle kernels done, [2] copy
 * out done, [3] field update done (the reference's Timers, src/Tools/Timers.cpp). */
int sg_sim_stream_timing( sg_sim *sim, float *ms );

/* Adds a Gaussian 2D laser injected through the Silver-Mueller condition on xmin
 * (LaserGaussian2D, src/Python/pyprofiles.py:507; ElectroMagnBC2D_SM::apply,
 * src/ElectroMagnBC/ElectroMagnBC2D_SM.cpp:118).  p = {a0, omega, waist, focus_x,
 * focus_y, polarization_phi, ellipticity, phase_offset, t_start, t_duration, t_center,
 * t_fwhm, t_order} (time envelope tgaussian).  The step k (0-based, counted from
 * creation) applies it at time (k + 1.5) dt, the reference's time_dual of iteration k+1.
 * Needs a 2D grid with an open x axis; at most 4 lasers. */
int sg_sim_add_laser_gaussian2d( sg_sim *sim, const double *params );

/* Segment re-layouts so far (each follows a step in which some tile's segment filled
 * up) and the particles that went through the spill list.  No reference counterpart:
 * the reference re-sorts every step. */
int sg_sim_layout_stats( sg_sim *sim, int64_t *relayouts, int64_t *spilled );

/* Moving window (SimWindow, src/MovWindow/SimWindow.cpp:30-96; shift :98-560).  At
 * the end of step k, when ((k + 1.5) dt - time_start) velocity_x > x_moved, the
 * window moves shift_cells cells towards +x (the reference's patch width along x):
 * that step skips its x boundaries; then every field moves shift_cells cells
 * towards xmin with zeros in the fresh cells, Silver-Mueller is applied on xmin,
 * lasers are switched off for good, particles that fall below x = 0 are removed,
 * the rest follow the window (positions stay window-relative: the reference keeps
 * absolute ones), the fresh cells are filled from each species' profile
 * (sg_sim_set_species_profile), and x_moved grows by shift_cells dx.  Needs a 2D
 * grid with an open x axis. */
int sg_sim_set_moving_window( sg_sim *sim, double time_start, double velocity_x, int shift_cells );
/* Cells and distance moved so far, and the number of shifts. */
int sg_sim_window_state( sg_sim *sim, int64_t *n_moved, double *x_moved, int64_t *shifts );

/* Density profile of a species for particle creation (ParticleCreator::create,
 * src/Particles/ParticleCreator.cpp:110-345): profile = {n0, x_vacuum, x_slope1,
 * x_plateau, x_slope2}, the reference's trapezoidal profile along x
 * (src/Profiles/Function.cpp:291-314) evaluated at absolute cell centres; ppc = c^ndim
 * particles per cell at regular positions (createPosition, :661-667); weight
 * n dV / ppc (createWeight, :933-939); momenta zero when temperature == 0, else
 * sqrt(temperature) times standard normals from a counter-based generator keyed on
 * (seed, absolute cell, particle). */
int sg_sim_set_species_profile( sg_sim *sim, int species, const double *profile, int ppc, double temperature,
                                uint64_t seed );
/* Creates the particles of the species' profile in window cells [x0_cell, x1_cell)
 * x every cell along y (z), as the reference does for its initial plasma. */
int sg_sim_fill_species( sg_sim *sim, int species, int x0_cell, int x1_cell );

/* Monte-Carlo radiation reaction of a species inside the resident step (2D mixed form):
 * before each push (Species::dynamics, src/Species/Species.cpp:583-640) every particle of
 * the species gets its E and B_m by the order-2 gather and one FP32-arithmetic pass of
 * RadiationMonteCarlo::operator() (sg_rad_tables_set_fp32_math) with `tables`, and with
 * the network `mlp` (may be NULL; validated) where its validation passed.  The species
 * then carries an optical depth per particle (starting spent, -1).  The random stream of
 * the particle in buffer slot o at step k is (seed, o, k): not the operator pass's.
 * Photons are tallied, not created.  The tables and the network must outlive the
 * simulation or the next call. */
int sg_sim_set_species_radiation( sg_sim *sim, int species, const sg_rad_tables *tables, const sg_mlp *mlp,
                                  uint32_t seed );
/* Radiated energy (sum of w (gamma_before - gamma_after)) and number of emissions of a
 * radiating species since sg_sim_set_species_radiation. */
int sg_sim_radiation_stats( sg_sim *sim, int species, double *radiated, unsigned long long *emissions );

/* Macro-photons of a radiating species in the resident step, as a species whose
 * radiation_photon_species is set (RadiationMonteCarlo.cpp:425-545): an emission whose
 * photon gamma is at least gamma_threshold, while the particle has made fewer than
 * max_emissions photon groups in the step, appends `sampling` photons (weight w /
 * sampling, momentum photon_gamma p / |p| after the recoil, chi, tau = -1) at the
 * particle's position to a device store of `capacity` photons, and its energy is not
 * added to the radiated tally.  Each step then pushes every stored photon
 * (PusherPhoton, src/Pusher/PusherPhoton.cpp:30-85: x += dt p / |p|, wrapped on periodic
 * axes; on an open axis it keeps going, and a moving window does not shift it).  Photons
 * past the capacity are counted, not stored.  capacity 0 removes the store.  Call after
 * sg_sim_set_species_radiation. */
int sg_sim_set_species_photons( sg_sim *sim, int species, int sampling, double gamma_threshold, int max_emissions,
                                int64_t capacity );

/* The photons wanted so far (*count; may pass the capacity) and host copies of the n =
 * min(count, capacity) stored ones: pos[d * n + k] (x, y), mom[c * n + k], weight[k],
 * chi[k], tau[k].  Any output may be NULL. */
int sg_sim_get_photons( sg_sim *sim, int species, int64_t *count, double *pos, double *mom, double *weight,
                        double *chi, double *tau );

/* Device time of the last sg_sim_step call split by stage (ms): particles, fold,
 * maxwell, total; and the number of kernel launches per step. */
int sg_sim_last_timing( sg_sim *sim, double *ms_particles, double *ms_fields, double *ms_total, int *launches_per_step );

/* Sets the stream the simulation runs on (default: a stream it creates). */
int sg_sim_set_stream( sg_sim *sim, sg_stream_t stream );

/* ---- Monte-Carlo radiation reaction ---- */


/* Uploads the radiation tables (host arrays, FP64) in the reference's conventions
 * (src/Radiation/Table.cpp:77-110; RadiationTables::initialization,
 * src/Radiation/RadiationTables.cpp:41-200): integfochi[n_integ] on log10-spaced
 * particle chi in [integ_min, integ_max]; xi[n_chi * n_ph] the cumulative photon-chi
 * distribution per particle chi in [xi_min, xi_max]; axis1_min[n_chi] the log10 of
 * each row's smallest photon chi.  factors = {factor_dNph_dt, factor_classical_radiated_power,
 * inv_norm_E_Schwinger, minimum_chi_continuous, minimum_chi_discontinuous}. */
int sg_rad_tables_create( const double *integ, int n_integ, double integ_min, double integ_max, const double *xi,
                          int n_chi, int n_ph, double xi_min, double xi_max, const double *axis1_min,
                          const double *factors, sg_rad_tables **out );
int sg_rad_tables_destroy( sg_rad_tables *tables );

/* Arithmetic of the Monte-Carlo passes that use these tables: 0 (default) FP64, as the
 * reference; 1 FP32 for the table lookups, the optical-depth draw and the continuous
 * loss (chi, gamma, times and momenta stay FP64).  FP64 runs at a small fraction of the
 * FP32 rate on GB300; the FP32 pass draws the same random numbers and agrees with the
 * FP64 pass statistically, not bit for bit. */
int sg_rad_tables_set_fp32_math( sg_rad_tables *tables, int on );

/* Inverse CDF (particle chi, xi) -> photon chi: replaces
 * RadiationTables::computeRandomPhotonChiWithInterpolation (RadiationTables.cpp:375). */
int sg_rad_photon_chi( const sg_rad_tables *tables, int64_t n, const double *chi, const double *xi, double *out,
                       sg_stream_t stream );

/* dN_photon/dt: replaces RadiationTables::computePhotonProductionYield (RadiationTables.cpp:225). */
int sg_rad_production_yield( const sg_rad_tables *tables, int64_t n, const double *chi, const double *gamma,
                             double *out, sg_stream_t stream );

/* One Monte-Carlo radiation pass over n particles (device arrays: mom[3n] updated,
 * weight[n], tau[n] optical depth updated, chi_out[n] optional: chi of the final
 * momentum, RadiationMonteCarlo.cpp:642-655; Epart/Bpart[3n] the interpolated fields):
 * replaces RadiationMonteCarlo::operator() (src/Radiation/RadiationMonteCarlo.cpp:62,
 * called from Species.cpp:615) with the emitted energy tallied instead of macro-photons
 * created.  Particle p draws from its own counter-based stream (seed, first_id + p,
 * step): xorshift32 from that state with x / 2^32 per draw, the stream a reference
 * Random seeded with the same state gives (src/Tools/Random.h:74-75).  radiated (device double) and
 * n_emissions (device) are accumulated.  mlp: NULL for the table inverse CDF, or a
 * validated network (sg_mlp_validate) used wherever its checked error is within
 * tolerance. */
int sg_rad_monte_carlo( const sg_rad_tables *tables, const sg_mlp *mlp, int64_t n, double dt, double mass,
                        double charge, double *mom, const double *weight, double *tau, double *chi_out,
                        const double *Epart, const double *Bpart, uint32_t seed, uint32_t first_id, uint32_t step,
                        double *radiated, unsigned long long *n_emissions, sg_stream_t stream );

/* The same pass creating macro-photons (RadiationMonteCarlo.cpp:425-545), as a species
 * with radiation_photon_species set: an emission whose photon gamma is at least
 * gamma_threshold (radiation_photon_gamma_threshold), while the particle has made
 * fewer than max_emissions photon groups (radiation_max_emissions) in this call,
 * appends `sampling` photons (radiation_photon_sampling) at the particle's position
 * (pos[d * n + i], ndim rows) with momentum photon_gamma p / |p| (p after the recoil),
 * weight w / sampling, chi = the photon's chi and tau = -1; the energy of such an
 * emission is not added to *radiated.  Photon k goes to ph_pos[d * photon_capacity + k],
 * ph_mom[c * photon_capacity + k], ph_weight[k], ph_chi[k], ph_tau[k] in the order the
 * slots are taken (atomically: not the particle order); *n_photons (device) is
 * incremented by the number of photons wanted, and slots at or past photon_capacity are
 * not written.  A capacity of n * max_emissions * sampling never overflows, like the
 * reference's per-particle GPU buffers. */
int sg_rad_monte_carlo_photons( const sg_rad_tables *tables, const sg_mlp *mlp, int ndim, int64_t n, double dt,
                                double mass, double charge, const double *pos, double *mom, const double *weight,
                                double *tau, double *chi_out, const double *Epart, const double *Bpart,
                                uint32_t seed, uint32_t first_id, uint32_t step, int sampling,
                                double gamma_threshold, int max_emissions, int64_t photon_capacity, double *ph_pos,
                                double *ph_mom, double *ph_weight, double *ph_chi, double *ph_tau,
                                unsigned long long *n_photons, double *radiated, unsigned long long *n_emissions,
                                sg_stream_t stream );

/* Rectilinear photon push (PusherPhoton::operator(), src/Pusher/PusherPhoton.cpp:30):
 * invgf[i] = 1 / |p_i| (optional), pos[d * n + i] += dt p_d invgf.  Device pointers. */
int sg_push_photons( int ndim, int64_t n, double dt, double *pos, const double *mom, double *invgf,
                     sg_stream_t stream );

/* The learned inverse CDF: an FP32 MLP 2 -> hidden -> hidden -> 1 (tanh) from
 * (log10 chi normalised to [log10_chi_min, log10_chi_max], xi) to
 * log10(photon chi / chi) / 8.  Trained on the GPU (forward, backward, batch
 * gradient reduction, Adam) on samples whose targets are the table inverse CDF. */
int sg_mlp_create( int hidden, uint32_t seed, double log10_chi_min, double log10_chi_max, sg_mlp **out );
int sg_mlp_destroy( sg_mlp *mlp );
int sg_mlp_nparams( const sg_mlp *mlp, int *n );
int sg_mlp_get_params( const sg_mlp *mlp, float *host );
int sg_mlp_set_params( sg_mlp *mlp, const float *host );
/* Gradient of the mean-squared loss over a host batch (inputs[2B] normalised, targets[B]). */
int sg_mlp_gradients( sg_mlp *mlp, int batch, const float *inputs, const float *targets, float *grad, float *loss );
/* steps of Adam on fresh table samples of the given batch size; final_loss optional. */
int sg_mlp_train( sg_mlp *mlp, const sg_rad_tables *tables, int steps, int batch, float lr, uint32_t seed,
                  float *final_loss, sg_stream_t stream );
/* Measures max |log10 mlp - log10 table| on per_bin^2 points of each of the
 * n_chi_bins x n_xi_bins bins and masks (falls back to the table on) every bin
 * above tol.  err_out[n_chi_bins * n_xi_bins] optional. */
int sg_mlp_validate( sg_mlp *mlp, const sg_rad_tables *tables, int n_chi_bins, int n_xi_bins, int per_bin,
                     float tol, float *err_out, int *n_masked );
/* Network inverse CDF alone (no fallback), device arrays.  A 64-wide network runs its
 * 64 x 64 layer on the tensor cores (mma.sync, FP16 operands, FP32 accumulation); other
 * widths, and sg_mlp_photon_chi_fp32 for every width, run on the FP32 cores.  No
 * reference counterpart: the reference has the table only
 * (RadiationTables::computeRandomPhotonChiWithInterpolation, RadiationTables.cpp:375). */
int sg_mlp_photon_chi( const sg_mlp *mlp, int64_t n, const double *chi, const double *xi, double *out,
                       sg_stream_t stream );
int sg_mlp_photon_chi_fp32( const sg_mlp *mlp, int64_t n, const double *chi, const double *xi, double *out,
                            sg_stream_t stream );

#ifdef __cplusplus
}
#endif

#endif /* SMILEI_GB300_H */
