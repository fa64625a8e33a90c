// Per-cell particle sort (drop-in for Species::sortParticles / SpeciesV::sortParticles).
//
// key  = exact int32 cell key from the positions (SpeciesV::computeParticleCellKeys,
//        src/Species/SpeciesV.cpp:766-857)
// bins = counts -> exclusive prefix sum -> first_index / last_index
//        (SpeciesV.cpp:645-652)
// order: a counting sort.  Slots inside a cell are handed out by atomics, then
//        each cell's slot list is re-ordered by original index so the result is
//        stable and deterministic; every property array is then gathered.

#include "common.cuh"
#include "scan.cuh"

#include <cmath>
#include <mutex>

namespace sg {
namespace {

struct KeyGeom {
    int ndim;
    int len[3];     // patch_size + 1 nodes per dimension
    double mn[3];   // round(xmin/dx)
    double dxi[3];
};

__global__ void k_cell_keys( KeyGeom g, int64_t n, const double *__restrict__ x, const double *__restrict__ y,
                             const double *__restrict__ z, int *__restrict__ keys, int *__restrict__ count,
                             int *__restrict__ status )
{
    const int64_t p = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x;
    if( p >= n ) return;
    int key = 0;
    bool ok = true;
    for( int d = 0; d < g.ndim; d++ ) {
        const double xd = d == 0 ? x[p] : ( d == 1 ? y[p] : z[p] );
        const int c = ( int )( round( xd * g.dxi[d] ) - g.mn[d] );
        if( c < 0 || c >= g.len[d] ) ok = false;
        key = key * g.len[d] + c;
    }
    if( !ok ) {
        atomicCAS( status, 0, SG_ERR_BOUNDS );
        key = 0;
    }
    keys[p] = key;
    atomicAdd( &count[key], 1 );
}

__global__ void k_bins( int ncell, const int64_t *__restrict__ off, const int *__restrict__ count,
                        int *__restrict__ first, int *__restrict__ last, int *__restrict__ fill )
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if( c >= ncell ) return;
    first[c] = ( int )off[c];
    last[c] = ( int )( off[c] + count[c] );
    fill[c] = ( int )off[c];
}

__global__ void k_slots( int64_t n, const int *__restrict__ keys, int *__restrict__ fill, int *__restrict__ perm )
{
    const int64_t p = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x;
    if( p >= n ) return;
    const int slot = atomicAdd( &fill[keys[p]], 1 );
    perm[slot] = ( int )p;
}

// One thread per cell: insertion sort of the cell's original indices.
__global__ void k_stable_cells( int ncell, const int *__restrict__ first, const int *__restrict__ last,
                                int *__restrict__ perm )
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if( c >= ncell ) return;
    const int a = first[c], b = last[c];
    for( int i = a + 1; i < b; i++ ) {
        const int v = perm[i];
        int j = i - 1;
        while( j >= a && perm[j] > v ) {
            perm[j + 1] = perm[j];
            j--;
        }
        perm[j + 1] = v;
    }
}

template <class T>
__global__ void k_gather( int64_t n, const int *__restrict__ perm, const T *__restrict__ src, T *__restrict__ dst )
{
    const int64_t q = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x;
    if( q < n ) dst[q] = src[perm[q]];
}

__global__ void k_permute_keys( int64_t n, const int *__restrict__ perm, const int *__restrict__ keys,
                                int *__restrict__ out )
{
    const int64_t q = ( int64_t )blockIdx.x * blockDim.x + threadIdx.x;
    if( q < n ) out[q] = keys[perm[q]];
}

// The whole sort on caller-provided scratch.  Returns the device status word in *h_status.
int sort_with_scratch( const KeyGeom &g, int ncell, int64_t npart, double *const *dprops, int n_dprops, short *charge,
                       int *first_index, int *last_index, int *cell_keys, int64_t *off, int64_t *scan_tmp, int *keys,
                       int *perm, int *count, int *fill, int *status, double *tmp, cudaStream_t s, int *h_status )
{
    SG_CUDA_TRY( cudaMemsetAsync( count, 0, ncell * sizeof( int ), s ) );
    SG_CUDA_TRY( cudaMemsetAsync( status, 0, sizeof( int ), s ) );
    const unsigned gp = grid_for( npart, 256 ), gc = grid_for( ncell, 256 );
    k_cell_keys<<<gp, 256, 0, s>>>( g, npart, dprops[0], g.ndim > 1 ? dprops[1] : nullptr,
                                    g.ndim > 2 ? dprops[2] : nullptr, keys, count, status );
    SG_LAUNCH_CHECK( "k_cell_keys" );
    int st = exclusive_scan<int>( count, ncell, off, scan_tmp, s );
    if( st ) return st;
    k_bins<<<gc, 256, 0, s>>>( ncell, off, count, first_index, last_index, fill );
    SG_LAUNCH_CHECK( "k_bins" );
    k_slots<<<gp, 256, 0, s>>>( npart, keys, fill, perm );
    SG_LAUNCH_CHECK( "k_slots" );
    k_stable_cells<<<gc, 256, 0, s>>>( ncell, first_index, last_index, perm );
    SG_LAUNCH_CHECK( "k_stable_cells" );
    for( int k = 0; k < n_dprops; k++ ) {
        k_gather<double><<<gp, 256, 0, s>>>( npart, perm, dprops[k], tmp );
        SG_LAUNCH_CHECK( "k_gather" );
        SG_CUDA_TRY( cudaMemcpyAsync( dprops[k], tmp, npart * sizeof( double ), cudaMemcpyDeviceToDevice, s ) );
    }
    if( charge ) {
        short *t16 = reinterpret_cast<short *>( tmp );
        k_gather<short><<<gp, 256, 0, s>>>( npart, perm, charge, t16 );
        SG_LAUNCH_CHECK( "k_gather" );
        SG_CUDA_TRY( cudaMemcpyAsync( charge, t16, npart * sizeof( short ), cudaMemcpyDeviceToDevice, s ) );
    }
    if( cell_keys ) {
        k_permute_keys<<<gp, 256, 0, s>>>( npart, perm, keys, cell_keys );
        SG_LAUNCH_CHECK( "k_permute_keys" );
    }
    SG_CUDA_TRY( cudaMemcpyAsync( h_status, status, sizeof( int ), cudaMemcpyDeviceToHost, s ) );
    return SG_OK;
}

} // namespace
} // namespace sg

using namespace sg;

extern "C" int sg_sort_particles( int ndim, const int *patch_size, const double *xmin, const double *cell_length,
                                  int64_t npart, double *const *dprops, int n_dprops, short *charge,
                                  int *first_index, int *last_index, int *cell_keys, sg_stream_t stream )
{
    SG_REQUIRE( ndim >= 1 && ndim <= 3, "ndim must be 1..3" );
    SG_REQUIRE( patch_size && xmin && cell_length, "NULL geometry" );
    SG_REQUIRE( npart >= 0 && npart < ( int64_t )1 << 31, "npart out of range" );
    SG_REQUIRE( n_dprops >= ndim, "dprops must start with the ndim position arrays" );
    SG_REQUIRE( dprops && first_index && last_index, "NULL array" );
    KeyGeom g{};
    g.ndim = ndim;
    int64_t ncell64 = 1;
    for( int d = 0; d < ndim; d++ ) {
        SG_REQUIRE( patch_size[d] > 0 && cell_length[d] > 0.0, "bad patch size / cell length in dim %d", d );
        g.len[d] = patch_size[d] + 1;
        g.dxi[d] = 1.0 / cell_length[d];
        g.mn[d] = std::round( xmin[d] * g.dxi[d] );
        ncell64 *= g.len[d];
    }
    SG_REQUIRE( ncell64 < ( int64_t )1 << 31, "too many cells" );
    const int ncell = ( int )ncell64;
    cudaStream_t s = as_stream( stream );
    if( npart == 0 ) {
        SG_CUDA_TRY( cudaMemsetAsync( first_index, 0, ncell * sizeof( int ), s ) );
        SG_CUDA_TRY( cudaMemsetAsync( last_index, 0, ncell * sizeof( int ), s ) );
        return SG_OK;
    }
    // Scratch: offsets + scan scratch (int64), keys/perm/count/fill/status (int32), one gather buffer.
    const int64_t scan_elems = scan_scratch_elems( ncell );
    const size_t n_i64 = ( size_t )ncell + ( size_t )scan_elems + 8;
    const size_t n_int = ( size_t )npart * 2 + ( size_t )ncell * 2 + 64;
    const size_t off_int = n_i64 * 8;
    const size_t off_tmp = ( ( off_int + n_int * 4 + 255 ) / 256 ) * 256;
    const size_t bytes = off_tmp + ( size_t )npart * 8;
    char *scratch = nullptr;
    SG_CUDA_TRY( cudaMallocAsync( &scratch, bytes, s ) );
    int64_t *off = reinterpret_cast<int64_t *>( scratch );
    int64_t *scan_tmp = off + ncell;
    int *keys = reinterpret_cast<int *>( scratch + off_int );
    int *perm = keys + npart;
    int *count = perm + npart;
    int *fill = count + ncell;
    int *status = fill + ncell;
    double *tmp = reinterpret_cast<double *>( scratch + off_tmp );
    int h_status = 0;
    int rc = sort_with_scratch( g, ncell, npart, dprops, n_dprops, charge, first_index, last_index, cell_keys, off,
                                scan_tmp, keys, perm, count, fill, status, tmp, s, &h_status );
    cudaError_t fe = cudaFreeAsync( scratch, s );
    if( rc ) return rc;
    if( fe != cudaSuccess ) return cuda_fail( fe, "cudaFreeAsync", __FILE__, __LINE__ );
    SG_CUDA_TRY( cudaStreamSynchronize( s ) );
    if( h_status ) return set_error( h_status, "a particle lies outside the patch's node lattice" );
    return SG_OK;
}

// ---- per-cell sort without allocation --------------------------------------
//
// Some callers cannot call cudaMalloc: code running while a CUDA graph is being
// captured in global mode, where allocation calls are refused; hosts that hand
// the library a fixed device-memory budget and forbid it to grow; and real-time
// loops in which an allocation's implicit synchronisation or latency is not
// acceptable.  sg_sort_particles_noalloc serves them with the same sort on a
// scratch area that is part of the library's own device image: a file-scope
// __device__ array of SG_SORT_NOALLOC_SCRATCH_BYTES, present on every GPU that
// loads the library until the process exits.  The host learns its device
// address once per device through cudaGetSymbolAddress (the array's name in
// host code is only a host-side stand-in and must never be passed to a kernel).

namespace sg {
namespace {

static __device__ __align__( 256 ) unsigned char g_sort_scratch[SG_SORT_NOALLOC_SCRATCH_BYTES];

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_scratch_mu;
void *g_scratch_dev[NOALLOC_MAX_DEVICES] = {};

// Device address of g_sort_scratch on the current device, looked up on the first
// call made with that device current.
int noalloc_scratch( char **out )
{
    int dev = -1;
    SG_CUDA_TRY( cudaGetDevice( &dev ) );
    if( dev < 0 || dev >= NOALLOC_MAX_DEVICES ) return set_error( SG_ERR_ARG, "device ordinal %d not supported", dev );
    std::lock_guard<std::mutex> lock( g_scratch_mu );
    if( !g_scratch_dev[dev] ) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress( &p, g_sort_scratch );
        if( e != cudaSuccess ) return cuda_fail( e, "cudaGetSymbolAddress(g_sort_scratch)", __FILE__, __LINE__ );
        g_scratch_dev[dev] = p;
    }
    *out = static_cast<char *>( g_scratch_dev[dev] );
    return SG_OK;
}

} // namespace
} // namespace sg

extern "C" int sg_sort_particles_noalloc( int ndim, const int *patch_size, const double *xmin,
                                          const double *cell_length, int64_t npart, double *const *dprops,
                                          int n_dprops, short *charge, int *first_index, int *last_index,
                                          int *cell_keys, sg_stream_t stream )
{
    SG_REQUIRE( ndim >= 1 && ndim <= 3, "ndim must be 1..3" );
    SG_REQUIRE( patch_size && xmin && cell_length, "NULL geometry" );
    SG_REQUIRE( npart >= 0, "npart out of range" );
    SG_REQUIRE( npart <= SG_SORT_NOALLOC_MAX_PARTICLES,
                "sg_sort_particles_noalloc: %lld particles exceed its fixed scratch limit of %d; use sg_sort_particles",
                ( long long )npart, SG_SORT_NOALLOC_MAX_PARTICLES );
    SG_REQUIRE( n_dprops >= ndim, "dprops must start with the ndim position arrays" );
    SG_REQUIRE( dprops && first_index && last_index, "NULL array" );
    KeyGeom g{};
    g.ndim = ndim;
    int64_t ncell64 = 1;
    for( int d = 0; d < ndim; d++ ) {
        SG_REQUIRE( patch_size[d] > 0 && cell_length[d] > 0.0, "bad patch size / cell length in dim %d", d );
        g.len[d] = patch_size[d] + 1;
        g.dxi[d] = 1.0 / cell_length[d];
        g.mn[d] = std::round( xmin[d] * g.dxi[d] );
        ncell64 *= g.len[d];
    }
    SG_REQUIRE( ncell64 <= SG_SORT_NOALLOC_MAX_CELLS,
                "sg_sort_particles_noalloc: %lld cells exceed its fixed scratch limit of %d; use sg_sort_particles",
                ( long long )ncell64, SG_SORT_NOALLOC_MAX_CELLS );
    const int ncell = ( int )ncell64;
    // same scratch layout as sg_sort_particles, carved from the static array
    const int64_t scan_elems = scan_scratch_elems( ncell );
    const size_t n_i64 = ( size_t )ncell + ( size_t )scan_elems + 8;
    const size_t n_int = ( size_t )npart * 2 + ( size_t )ncell * 2 + 64;
    const size_t off_int = n_i64 * 8;
    const size_t off_tmp = ( ( off_int + n_int * 4 + 255 ) / 256 ) * 256;
    const size_t bytes = off_tmp + ( size_t )npart * 8;
    SG_REQUIRE( bytes <= ( size_t )SG_SORT_NOALLOC_SCRATCH_BYTES,
                "sg_sort_particles_noalloc: needs %zu scratch bytes, more than its %d", bytes,
                SG_SORT_NOALLOC_SCRATCH_BYTES );
    char *scratch = nullptr;
    int rc = noalloc_scratch( &scratch );
    if( rc ) return rc;
    cudaStream_t s = as_stream( stream );
    if( npart == 0 ) {
        SG_CUDA_TRY( cudaMemsetAsync( first_index, 0, ncell * sizeof( int ), s ) );
        SG_CUDA_TRY( cudaMemsetAsync( last_index, 0, ncell * sizeof( int ), s ) );
        return SG_OK;
    }
    int64_t *off = reinterpret_cast<int64_t *>( scratch );
    int64_t *scan_tmp = off + ncell;
    int *keys = reinterpret_cast<int *>( scratch + off_int );
    int *perm = keys + npart;
    int *count = perm + npart;
    int *fill = count + ncell;
    int *status = fill + ncell;
    double *tmp = reinterpret_cast<double *>( scratch + off_tmp );
    // The array keeps the previous call's contents: the per-cell counts and the
    // status word are cleared inside sort_with_scratch; every other region is
    // fully written before it is read.
    int h_status = 0;
    rc = sort_with_scratch( g, ncell, npart, dprops, n_dprops, charge, first_index, last_index, cell_keys, off,
                            scan_tmp, keys, perm, count, fill, status, tmp, s, &h_status );
    if( rc ) {
        // work queued before the failure may still use the shared array: let it end
        // before the caller retries (perhaps on another stream)
        cudaStreamSynchronize( s );
        cudaGetLastError();
        return rc;
    }
    SG_CUDA_TRY( cudaStreamSynchronize( s ) );
    if( h_status ) return set_error( h_status, "a particle lies outside the patch's node lattice" );
    return SG_OK;
}
