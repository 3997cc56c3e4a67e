/* No-op stand-in for the HDF5 API: the reference's field/distribution
 * writers compile against it but write nothing. Used only to build the
 * reference CPU path as a test oracle. */
#pragma once
typedef long hid_t;
typedef int herr_t;
typedef unsigned long long hsize_t;
#define H5P_DATASET_XFER 0
#define H5P_FILE_ACCESS 0
#define H5P_DEFAULT 0
#define H5F_ACC_TRUNC 0
#define H5F_ACC_RDONLY 0
#define H5T_NATIVE_DOUBLE 0
#define H5S_SELECT_SET 0
#define H5FD_MPIO_COLLECTIVE 0
template <class... A> inline long mlbm_h5_noop(A...) { return 0; }
#define H5Pcreate mlbm_h5_noop
#define H5Pclose mlbm_h5_noop
#define H5Fclose mlbm_h5_noop
#define H5Fcreate mlbm_h5_noop
#define H5Fopen mlbm_h5_noop
#define H5Screate_simple mlbm_h5_noop
#define H5Sclose mlbm_h5_noop
#define H5Dcreate mlbm_h5_noop
#define H5Dcreate2 mlbm_h5_noop
#define H5Dopen mlbm_h5_noop
#define H5Dopen2 mlbm_h5_noop
#define H5Dclose mlbm_h5_noop
#define H5Dget_space mlbm_h5_noop
#define H5Dwrite mlbm_h5_noop
#define H5Dread mlbm_h5_noop
#define H5Sselect_hyperslab mlbm_h5_noop
#define H5Pset_dxpl_mpio mlbm_h5_noop
#define H5Pset_fapl_mpio mlbm_h5_noop
