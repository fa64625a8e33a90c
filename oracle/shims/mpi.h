/* Test-infrastructure header: a single-rank stand-in for <mpi.h>.
 *
 * It exists only so that a handful of the reference's operator sources
 * (interpolators, pushers, projectors, Yee solvers, radiation tables) can be
 * compiled directly from the reference tree into the oracle executable
 * oracle/_ref/ref_ops.  Those operators make no MPI calls; their headers only
 * name MPI types and a few functions.  Every function here is a local no-op
 * or a local copy (one rank), so the operators behave exactly as in a 1-rank
 * reference run.  Nothing in the product links against this header.
 */
#ifndef SG_ORACLE_MPI_SHIM_H
#define SG_ORACLE_MPI_SHIM_H
#include <cstring>
#include <cstdlib>
#include <cstdint>
#include <chrono>

typedef int  MPI_Comm;
typedef int  MPI_Request;
typedef int  MPI_Datatype;
typedef int  MPI_Op;
typedef int  MPI_Info;
typedef long MPI_Aint;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD      1
#define MPI_STATUS_IGNORE   ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_IN_PLACE        ((void *)1)
#define MPI_PROC_NULL       (-2)
#define MPI_UNDEFINED       (-32766)
#define MPI_REQUEST_NULL    0
#define MPI_DATATYPE_NULL   0
#define MPI_INFO_NULL       0
#define MPI_TAG_UB          77
#define MPI_BSEND_OVERHEAD  96
#define MPI_THREAD_SINGLE     0
#define MPI_THREAD_FUNNELED   1
#define MPI_THREAD_SERIALIZED 2
#define MPI_THREAD_MULTIPLE   3
#define MPI_SUCCESS         0
#define MPI_MAX_PROCESSOR_NAME 64

enum { MPI_CHAR = 1, MPI_SHORT, MPI_INT, MPI_LONG, MPI_UNSIGNED, MPI_UNSIGNED_LONG,
       MPI_UNSIGNED_LONG_LONG, MPI_LONG_LONG, MPI_UINT64_T, MPI_DOUBLE, MPI_FLOAT,
       MPI_CXX_BOOL, MPI_C_BOOL, MPI_DOUBLE_INT, MPI_PACKED, MPI_BYTE, MPI_UNSIGNED_SHORT };
enum { MPI_SUM = 1, MPI_MAX, MPI_MIN, MPI_LOR, MPI_LAND, MPI_MAXLOC, MPI_MINLOC, MPI_PROD };

static inline size_t sg_mpi_type_size( MPI_Datatype t )
{
    switch( t ) {
        case MPI_CHAR: case MPI_PACKED: case MPI_CXX_BOOL: case MPI_C_BOOL: case MPI_BYTE: return 1;
        case MPI_SHORT: case MPI_UNSIGNED_SHORT: return 2;
        case MPI_INT: case MPI_UNSIGNED: case MPI_FLOAT: return 4;
        case MPI_DOUBLE_INT: return 16;
        default: return 8;
    }
}
static inline int sg_mpi_copy( const void *s, void *r, int n, MPI_Datatype t )
{
    if( s != MPI_IN_PLACE && s && r && s != r ) std::memmove( r, s, ( size_t )n * sg_mpi_type_size( t ) );
    return 0;
}
static inline double MPI_Wtime() { return std::chrono::duration<double>( std::chrono::steady_clock::now().time_since_epoch() ).count(); }
static inline int MPI_Init( int *, char *** ) { return 0; }
static inline int MPI_Init_thread( int *, char ***, int req, int *prov ) { *prov = req; return 0; }
static inline int MPI_Initialized( int *f ) { *f = 1; return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Abort( MPI_Comm, int c ) { std::exit( c ); }
static inline int MPI_Comm_rank( MPI_Comm, int *r ) { *r = 0; return 0; }
static inline int MPI_Comm_size( MPI_Comm, int *s ) { *s = 1; return 0; }
static inline int MPI_Comm_dup( MPI_Comm c, MPI_Comm *n ) { *n = c; return 0; }
static inline int MPI_Comm_free( MPI_Comm * ) { return 0; }
static inline int MPI_Comm_split( MPI_Comm c, int, int, MPI_Comm *n ) { *n = c; return 0; }
static inline int MPI_Comm_get_attr( MPI_Comm, int, void *v, int *f ) { static int ub = 1 << 30; static int *p = &ub; *( int ** )v = p; *f = 1; return 0; }
static inline int MPI_Get_processor_name( char *n, int *l ) { n[0] = 'x'; n[1] = 0; *l = 1; return 0; }
static inline int MPI_Barrier( MPI_Comm ) { return 0; }
static inline int MPI_Bcast( void *, int, MPI_Datatype, int, MPI_Comm ) { return 0; }
static inline int MPI_Allreduce( const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm ) { return sg_mpi_copy( s, r, n, t ); }
static inline int MPI_Reduce( const void *s, void *r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm ) { return sg_mpi_copy( s, r, n, t ); }
static inline int MPI_Scan( const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm ) { return sg_mpi_copy( s, r, n, t ); }
static inline int MPI_Exscan( const void *, void *, int, MPI_Datatype, MPI_Op, MPI_Comm ) { return 0; }
static inline int MPI_Allgather( const void *s, int n, MPI_Datatype t, void *r, int, MPI_Datatype, MPI_Comm ) { return sg_mpi_copy( s, r, n, t ); }
static inline int MPI_Allgatherv( const void *s, int n, MPI_Datatype t, void *r, const int *, const int *, MPI_Datatype, MPI_Comm ) { return sg_mpi_copy( s, r, n, t ); }
static inline int MPI_Gather( const void *s, int n, MPI_Datatype t, void *r, int, MPI_Datatype, int, MPI_Comm ) { return sg_mpi_copy( s, r, n, t ); }
static inline int MPI_Gatherv( const void *s, int n, MPI_Datatype t, void *r, const int *, const int *, MPI_Datatype, int, MPI_Comm ) { return sg_mpi_copy( s, r, n, t ); }
static inline int MPI_Alltoall( const void *s, int n, MPI_Datatype t, void *r, int, MPI_Datatype, MPI_Comm ) { return sg_mpi_copy( s, r, n, t ); }
static inline int MPI_Send( const void *, int, MPI_Datatype, int, int, MPI_Comm ) { return 0; }
static inline int MPI_Bsend( const void *, int, MPI_Datatype, int, int, MPI_Comm ) { return 0; }
static inline int MPI_Recv( void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status * ) { return 0; }
static inline int MPI_Isend( const void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *q ) { *q = 0; return 0; }
static inline int MPI_Irecv( void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *q ) { *q = 0; return 0; }
static inline int MPI_Sendrecv( const void *s, int n, MPI_Datatype t, int, int, void *r, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status * ) { return sg_mpi_copy( s, r, n, t ); }
static inline int MPI_Wait( MPI_Request *, MPI_Status * ) { return 0; }
static inline int MPI_Waitall( int, MPI_Request *, MPI_Status * ) { return 0; }
static inline int MPI_Test( MPI_Request *, int *f, MPI_Status * ) { *f = 1; return 0; }
static inline int MPI_Buffer_attach( void *, int ) { return 0; }
static inline int MPI_Buffer_detach( void *, int * ) { return 0; }
static inline int MPI_Get_address( const void *p, MPI_Aint *a ) { *a = ( MPI_Aint )p; return 0; }
static inline int MPI_Type_commit( MPI_Datatype * ) { return 0; }
static inline int MPI_Type_free( MPI_Datatype * ) { return 0; }
static inline int MPI_Type_contiguous( int, MPI_Datatype, MPI_Datatype *n ) { *n = MPI_DOUBLE; return 0; }
static inline int MPI_Type_vector( int, int, int, MPI_Datatype, MPI_Datatype *n ) { *n = MPI_DOUBLE; return 0; }
static inline int MPI_Type_create_struct( int, const int *, const MPI_Aint *, const MPI_Datatype *, MPI_Datatype *n ) { *n = MPI_DOUBLE; return 0; }
static inline int MPI_Type_create_subarray( int, const int *, const int *, const int *, int, MPI_Datatype, MPI_Datatype *n ) { *n = MPI_DOUBLE; return 0; }
static inline int MPI_Pack( const void *, int, MPI_Datatype, void *, int, int *, MPI_Comm ) { return 0; }
static inline int MPI_Unpack( const void *, int, int *, void *, int, MPI_Datatype, MPI_Comm ) { return 0; }
static inline int MPI_Pack_size( int n, MPI_Datatype t, MPI_Comm, int *s ) { *s = n * ( int )sg_mpi_type_size( t ); return 0; }

#endif
