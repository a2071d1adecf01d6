/* Test infrastructure (oracle): the subset of the HDF5 C API that the
 * reference's src/IO.cpp calls (file, dataspace, dataset and property-list
 * calls of save_instant_field), declared so that IO.cpp compiles unmodified
 * against the other shims; hdf5_stub.cpp gives them bodies that only check
 * their arguments and report success.  The time step never calls HDF5. */
#pragma once
#include <stdint.h>

#include "mpi.h"

typedef int64_t hid_t;
typedef int herr_t;
typedef unsigned long long hsize_t;
typedef enum { H5S_SELECT_SET = 0 } H5S_seloper_t;
typedef enum { H5FD_MPIO_INDEPENDENT = 0, H5FD_MPIO_COLLECTIVE = 1 } H5FD_mpio_xfer_t;

#define H5P_DEFAULT ((hid_t)0)
#define H5P_FILE_ACCESS ((hid_t)1)
#define H5P_DATASET_XFER ((hid_t)2)
#define H5T_NATIVE_DOUBLE ((hid_t)3)
#define H5F_ACC_TRUNC 2u

herr_t H5open(void);
herr_t H5close(void);
hid_t H5Pcreate(hid_t cls);
herr_t H5Pclose(hid_t plist);
herr_t H5Pset_fapl_mpio(hid_t fapl, MPI_Comm comm, MPI_Info info);
herr_t H5Pset_dxpl_mpio(hid_t dxpl, H5FD_mpio_xfer_t mode);
hid_t H5Fcreate(const char *name, unsigned flags, hid_t fcpl, hid_t fapl);
herr_t H5Fclose(hid_t file);
hid_t H5Screate_simple(int rank, const hsize_t *dims, const hsize_t *maxdims);
herr_t H5Sclose(hid_t space);
herr_t H5Sselect_hyperslab(hid_t space, H5S_seloper_t op, const hsize_t *start, const hsize_t *stride,
                           const hsize_t *count, const hsize_t *block);
hid_t H5Dcreate(hid_t loc, const char *name, hid_t type, hid_t space, hid_t lcpl, hid_t dcpl, hid_t dapl);
hid_t H5Dget_space(hid_t dset);
herr_t H5Dwrite(hid_t dset, hid_t mem_type, hid_t mem_space, hid_t file_space, hid_t plist, const void *buf);
herr_t H5Dclose(hid_t dset);
