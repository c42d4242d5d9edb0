/* Stand-in for the subset of the HDF5 1.8 C API that the reference solver uses.
 *
 * Test infrastructure only.  The reference includes <hdf5.h> unconditionally
 * (its partitioned-mesh and solution files are HDF5); this header plus
 * h5_stand_in.cpp give it a small object store with the same group / dataset /
 * attribute model, kept in memory while a file is open and saved to disk in a
 * private binary layout when it is closed.  The files it writes are therefore
 * readable only by programs linked against this stand-in, which is all the
 * reference build under oracle/refbuild needs: its decomposition step writes
 * the partitioned mesh and its solver step reads it back.
 *
 * Selections are whole-dataset (the reference always selects the full extent),
 * and numeric types convert on read and write as HDF5 does. */
#ifndef PCFD_REFBUILD_HDF5_H
#define PCFD_REFBUILD_HDF5_H

#include <cstddef>
#include <cstdint>

typedef int64_t hid_t;
typedef int herr_t;
typedef unsigned long long hsize_t;
typedef long long hssize_t;
typedef int htri_t;

#define H5P_DEFAULT ((hid_t)0)
#define H5S_ALL ((hid_t)0)

/* Native types are fixed ids; string types are handles made by H5Tcopy. */
#define H5T_NATIVE_CHAR ((hid_t)1001)
#define H5T_NATIVE_UCHAR ((hid_t)1002)
#define H5T_NATIVE_SHORT ((hid_t)1003)
#define H5T_NATIVE_USHORT ((hid_t)1004)
#define H5T_NATIVE_INT ((hid_t)1005)
#define H5T_NATIVE_UINT ((hid_t)1006)
#define H5T_NATIVE_LONG ((hid_t)1007)
#define H5T_NATIVE_ULONG ((hid_t)1008)
#define H5T_NATIVE_LLONG ((hid_t)1009)
#define H5T_NATIVE_ULLONG ((hid_t)1010)
#define H5T_NATIVE_FLOAT ((hid_t)1011)
#define H5T_NATIVE_DOUBLE ((hid_t)1012)
#define H5T_NATIVE_LDOUBLE ((hid_t)1013)
#define H5T_C_S1 ((hid_t)1020)

#define H5P_DATASET_XFER ((hid_t)2001)

#define H5F_ACC_RDONLY 0x0000u
#define H5F_ACC_RDWR 0x0001u
#define H5F_ACC_TRUNC 0x0002u
#define H5F_ACC_EXCL 0x0004u

typedef enum { H5S_NO_CLASS = -1, H5S_SCALAR = 0, H5S_SIMPLE = 1, H5S_NULL = 2 } H5S_class_t;
typedef enum { H5S_SELECT_NOOP = -1, H5S_SELECT_SET = 0, H5S_SELECT_OR = 1 } H5S_seloper_t;
typedef enum { H5_INDEX_UNKNOWN = -1, H5_INDEX_NAME = 0, H5_INDEX_CRT_ORDER = 1 } H5_index_t;
typedef enum { H5_ITER_UNKNOWN = -1, H5_ITER_INC = 0, H5_ITER_DEC = 1, H5_ITER_NATIVE = 2 } H5_iter_order_t;
typedef enum { H5G_UNKNOWN = -1, H5G_GROUP = 0, H5G_DATASET = 1, H5G_TYPE = 2, H5G_LINK = 3 } H5G_obj_t;

typedef struct { int type; int corder_valid; long long corder; int cset; } H5L_info_t;
typedef struct {
  unsigned long fileno[2];
  unsigned long objno[2];
  unsigned nlink;
  H5G_obj_t type;
  long long mtime;
  size_t linklen;
} H5G_stat_t;

typedef herr_t (*H5L_iterate_t)(hid_t group, const char* name, const H5L_info_t* info, void* op_data);
typedef herr_t (*H5E_auto1_t)(void* client_data);

herr_t H5Eset_auto1(H5E_auto1_t func, void* client_data);

hid_t H5Fcreate(const char* name, unsigned flags, hid_t fcpl, hid_t fapl);
hid_t H5Fopen(const char* name, unsigned flags, hid_t fapl);
herr_t H5Fclose(hid_t file);

hid_t H5Gopen2(hid_t loc, const char* name, hid_t gapl);
hid_t H5Gcreate2(hid_t loc, const char* name, hid_t lcpl, hid_t gcpl, hid_t gapl);
herr_t H5Gclose(hid_t group);
herr_t H5Gget_objinfo(hid_t loc, const char* name, int follow_link, H5G_stat_t* statbuf);
herr_t H5Literate(hid_t group, H5_index_t idx_type, H5_iter_order_t order, hsize_t* idx,
                  H5L_iterate_t op, void* op_data);

hid_t H5Screate(H5S_class_t type);
hid_t H5Screate_simple(int rank, const hsize_t* dims, const hsize_t* maxdims);
herr_t H5Sclose(hid_t space);
int H5Sget_simple_extent_ndims(hid_t space);
int H5Sget_simple_extent_dims(hid_t space, hsize_t* dims, hsize_t* maxdims);
herr_t H5Sselect_hyperslab(hid_t space, H5S_seloper_t op, const hsize_t* start, const hsize_t* stride,
                           const hsize_t* count, const hsize_t* block);

hid_t H5Tcopy(hid_t type);
herr_t H5Tset_size(hid_t type, size_t size);
size_t H5Tget_size(hid_t type);
herr_t H5Tclose(hid_t type);

hid_t H5Pcreate(hid_t cls);
herr_t H5Pset_buffer(hid_t plist, size_t size, void* tconv, void* bkg);
herr_t H5Pclose(hid_t plist);

hid_t H5Dopen2(hid_t loc, const char* name, hid_t dapl);
hid_t H5Dcreate2(hid_t loc, const char* name, hid_t type, hid_t space, hid_t lcpl, hid_t dcpl, hid_t dapl);
herr_t H5Dclose(hid_t dset);
hid_t H5Dget_type(hid_t dset);
hid_t H5Dget_space(hid_t dset);
herr_t H5Dread(hid_t dset, hid_t mem_type, hid_t mem_space, hid_t file_space, hid_t plist, void* buf);
herr_t H5Dwrite(hid_t dset, hid_t mem_type, hid_t mem_space, hid_t file_space, hid_t plist, const void* buf);

hid_t H5Acreate2(hid_t loc, const char* name, hid_t type, hid_t space, hid_t acpl, hid_t aapl);
hid_t H5Aopen(hid_t loc, const char* name, hid_t aapl);
herr_t H5Adelete(hid_t loc, const char* name);
herr_t H5Aclose(hid_t attr);
hid_t H5Aget_type(hid_t attr);
hid_t H5Aget_space(hid_t attr);
herr_t H5Aread(hid_t attr, hid_t mem_type, void* buf);
herr_t H5Awrite(hid_t attr, hid_t mem_type, const void* buf);

/* The 1.8 API's default (version 2) names. */
#define H5Gopen H5Gopen2
#define H5Gcreate H5Gcreate2
#define H5Dopen H5Dopen2
#define H5Dcreate H5Dcreate2
#define H5Acreate H5Acreate2

#endif
