#ifndef MXS_HDF5_HL_H
#define MXS_HDF5_HL_H
#include "hdf5.h"
#define H5LTset_attribute_double(...) ((herr_t)0)
#define H5LTset_attribute_int(...) ((herr_t)0)
#define H5LTset_attribute_string(...) ((herr_t)0)
#endif
