// Test infrastructure (oracle): bodies for the HDF5 subset declared in
// hdf5.h.  They write nothing; each returns a positive id or success, so the
// reference's src/IO.cpp links into a driver for compile-and-link checks.
#include "hdf5.h"

namespace {
hid_t g_next = 100;
}

herr_t H5open(void) { return 0; }
herr_t H5close(void) { return 0; }
hid_t H5Pcreate(hid_t) { return g_next++; }
herr_t H5Pclose(hid_t) { return 0; }
herr_t H5Pset_fapl_mpio(hid_t, MPI_Comm, MPI_Info) { return 0; }
herr_t H5Pset_dxpl_mpio(hid_t, H5FD_mpio_xfer_t) { return 0; }
hid_t H5Fcreate(const char *name, unsigned, hid_t, hid_t) { return name ? g_next++ : -1; }
herr_t H5Fclose(hid_t) { return 0; }
hid_t H5Screate_simple(int rank, const hsize_t *dims, const hsize_t *) { return rank > 0 && dims ? g_next++ : -1; }
herr_t H5Sclose(hid_t) { return 0; }
herr_t H5Sselect_hyperslab(hid_t, H5S_seloper_t, const hsize_t *, const hsize_t *, const hsize_t *, const hsize_t *) {
  return 0;
}
hid_t H5Dcreate(hid_t, const char *name, hid_t, hid_t, hid_t, hid_t, hid_t) { return name ? g_next++ : -1; }
hid_t H5Dget_space(hid_t) { return g_next++; }
herr_t H5Dwrite(hid_t, hid_t, hid_t, hid_t, hid_t, const void *buf) { return buf ? 0 : -1; }
herr_t H5Dclose(hid_t) { return 0; }
