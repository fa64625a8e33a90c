/* Test-infrastructure header: a declaration-only stand-in for <hdf5.h>.
 *
 * The reference's radiation tables and species headers include its HDF5
 * helpers; the operators compiled into oracle/_ref/ref_ops never write or read
 * a file, so every H5 call here is an inline no-op returning a positive id.
 * Nothing in the product uses this header.
 */
#ifndef SG_ORACLE_HDF5_SHIM_H
#define SG_ORACLE_HDF5_SHIM_H
#include <cstdint>

#define H5_HAVE_PARALLEL 1
#define H5_VERS_MAJOR 1
#define H5_VERS_MINOR 12
#define H5_VERS_RELEASE 0

typedef long long          hid_t;
typedef unsigned long long hsize_t;
typedef long long          hssize_t;
typedef int                herr_t;
typedef int                htri_t;
typedef int                H5D_layout_t;
typedef int                H5FD_mpio_xfer_t;
typedef int                H5T_class_t;
typedef herr_t ( *H5E_auto2_t )( hid_t, void * );

#define SG_H5_NOOP( name ) static inline long long name( ... ) { return 1; }
SG_H5_NOOP( H5Aclose ) SG_H5_NOOP( H5Acreate ) SG_H5_NOOP( H5Aexists ) SG_H5_NOOP( H5Aget_space )
SG_H5_NOOP( H5Aget_type ) SG_H5_NOOP( H5Aopen ) SG_H5_NOOP( H5Aopen_name ) SG_H5_NOOP( H5Aread )
SG_H5_NOOP( H5Awrite ) SG_H5_NOOP( H5Dclose ) SG_H5_NOOP( H5Dcreate ) SG_H5_NOOP( H5Dget_space )
SG_H5_NOOP( H5Dopen ) SG_H5_NOOP( H5Dread ) SG_H5_NOOP( H5Dset_extent ) SG_H5_NOOP( H5Dwrite )
SG_H5_NOOP( H5Eget_auto ) SG_H5_NOOP( H5Eget_num ) SG_H5_NOOP( H5Eprint2 ) SG_H5_NOOP( H5Eset_auto )
SG_H5_NOOP( H5Fclose ) SG_H5_NOOP( H5Fcreate ) SG_H5_NOOP( H5Fflush ) SG_H5_NOOP( H5Fopen )
SG_H5_NOOP( H5Gclose ) SG_H5_NOOP( H5Gcreate ) SG_H5_NOOP( H5Gopen ) SG_H5_NOOP( H5Gget_info )
SG_H5_NOOP( H5Lcreate_soft ) SG_H5_NOOP( H5Lexists ) SG_H5_NOOP( H5Literate ) SG_H5_NOOP( H5Oclose )
SG_H5_NOOP( H5Oopen ) SG_H5_NOOP( H5Oget_info ) SG_H5_NOOP( H5Pclose ) SG_H5_NOOP( H5Pcreate )
SG_H5_NOOP( H5Pget_dxpl_mpio ) SG_H5_NOOP( H5Pget_layout ) SG_H5_NOOP( H5Premove_filter )
SG_H5_NOOP( H5Pset_alignment ) SG_H5_NOOP( H5Pset_chunk ) SG_H5_NOOP( H5Pset_deflate )
SG_H5_NOOP( H5Pset_dxpl_mpio ) SG_H5_NOOP( H5Pset_fapl_mpio ) SG_H5_NOOP( H5Pset_layout )
SG_H5_NOOP( H5Pset_link_creation_order ) SG_H5_NOOP( H5Pset_create_intermediate_group )
SG_H5_NOOP( H5Pset_fill_time ) SG_H5_NOOP( H5Pset_alloc_time ) SG_H5_NOOP( H5Pset_meta_block_size )
SG_H5_NOOP( H5Pset_coll_metadata_write ) SG_H5_NOOP( H5Pset_all_coll_metadata_ops )
SG_H5_NOOP( H5Sclose ) SG_H5_NOOP( H5Screate ) SG_H5_NOOP( H5Screate_simple )
SG_H5_NOOP( H5Sget_simple_extent_dims ) SG_H5_NOOP( H5Sget_simple_extent_ndims )
SG_H5_NOOP( H5Sget_simple_extent_npoints ) SG_H5_NOOP( H5Sselect_hyperslab ) SG_H5_NOOP( H5Sselect_none )
SG_H5_NOOP( H5Sselect_all ) SG_H5_NOOP( H5Sselect_elements ) SG_H5_NOOP( H5Tclose ) SG_H5_NOOP( H5Tcopy )
SG_H5_NOOP( H5Tget_size ) SG_H5_NOOP( H5Tset_size ) SG_H5_NOOP( H5Tget_class ) SG_H5_NOOP( H5Tequal )
SG_H5_NOOP( H5Tcreate ) SG_H5_NOOP( H5Tinsert ) SG_H5_NOOP( H5Tget_native_type ) SG_H5_NOOP( H5Iget_name )
SG_H5_NOOP( H5Iis_valid ) SG_H5_NOOP( H5Iget_type ) SG_H5_NOOP( H5Oexists_by_name ) SG_H5_NOOP( H5Rcreate ) SG_H5_NOOP( H5Dget_type )
#undef SG_H5_NOOP

#define H5P_DEFAULT 0
#define H5S_ALL 0
#define H5S_UNLIMITED ( ( hsize_t )( -1 ) )
#define H5F_ACC_TRUNC 2
#define H5F_ACC_RDONLY 0
#define H5F_ACC_RDWR 1
#define H5F_SCOPE_GLOBAL 1
#define H5F_SCOPE_LOCAL 0
#define H5P_FILE_ACCESS 1
#define H5P_FILE_CREATE 2
#define H5P_DATASET_XFER 3
#define H5P_DATASET_CREATE 4
#define H5P_LINK_CREATE 5
#define H5P_GROUP_CREATE 6
#define H5P_DATASET_ACCESS 7
#define H5P_LINK_ACCESS 8
#define H5S_SELECT_SET 0
#define H5S_SELECT_OR 1
#define H5S_SCALAR 0
#define H5S_SIMPLE 1
#define H5S_NULL 2
#define H5FD_MPIO_COLLECTIVE 1
#define H5FD_MPIO_INDEPENDENT 0
#define H5D_CHUNKED 2
#define H5D_CONTIGUOUS 1
#define H5D_COMPACT 0
#define H5D_FILL_TIME_NEVER 2
#define H5D_ALLOC_TIME_EARLY 1
#define H5Z_FILTER_DEFLATE 1
#define H5P_CRT_ORDER_TRACKED 1
#define H5T_VARIABLE ( ( size_t )( -1 ) )
#define H5T_STRING 3
#define H5T_COMPOUND 6
#define H5E_DEFAULT 0
#define H5_INDEX_NAME 0
#define H5_INDEX_CRT_ORDER 1
#define H5_ITER_INC 0
#define H5_ITER_NATIVE 2
#define H5R_OBJECT 0
#define H5O_TYPE_GROUP 0
#define H5O_TYPE_DATASET 1
#define H5I_GROUP 2
#define H5I_DATASET 5
#define H5I_FILE 1
typedef int H5O_info_t;
typedef int H5G_info_t;
typedef int H5L_info_t;
typedef int H5L_info2_t;
typedef long long hobj_ref_t;

#define H5T_NATIVE_DOUBLE 11
#define H5T_NATIVE_FLOAT 12
#define H5T_NATIVE_INT 13
#define H5T_NATIVE_UINT 14
#define H5T_NATIVE_SHORT 15
#define H5T_NATIVE_USHORT 16
#define H5T_NATIVE_LONG 17
#define H5T_NATIVE_ULONG 18
#define H5T_NATIVE_LLONG 19
#define H5T_NATIVE_ULLONG 20
#define H5T_NATIVE_UINT64 21
#define H5T_NATIVE_INT64 22
#define H5T_NATIVE_UINT32 23
#define H5T_NATIVE_INT32 24
#define H5T_NATIVE_CHAR 25
#define H5T_NATIVE_UCHAR 26
#define H5T_NATIVE_HBOOL 27
#define H5T_NATIVE_B8 28
#define H5T_C_S1 29
#define H5T_STD_REF_OBJ 30
#define H5T_NATIVE_UINT8 31
#define H5T_NATIVE_INT8 32
#define H5T_NATIVE_SCHAR 33

#endif
