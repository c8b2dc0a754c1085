// Definitions for the no-op HDF5 stand-in (see H5Cpp.h).  Test infrastructure.
#include "H5Cpp.h"
const H5::DataType H5::PredType::NATIVE_DOUBLE;
const H5::DataType H5::PredType::NATIVE_ULLONG;
