/* Declarations-only stand-in for the HDF5 types the reference's headers name
 * (TEST INFRASTRUCTURE for oracle/ref.mk).  No HDF5 function is reachable on
 * the Henon-step path; any that is linked aborts (refshim.c). */
#ifndef CMCREF_SHIM_HDF5_H
#define CMCREF_SHIM_HDF5_H
typedef int herr_t;
typedef long long hid_t;
typedef unsigned long long hsize_t;
#define H5T_NATIVE_DOUBLE ((hid_t)1)
#define H5T_NATIVE_INT ((hid_t)2)
#define H5T_NATIVE_LONG ((hid_t)3)
#define H5T_C_S1 ((hid_t)4)
#define H5F_ACC_TRUNC 0
#define H5F_ACC_RDONLY 0
#define H5P_DEFAULT ((hid_t)0)
#endif
