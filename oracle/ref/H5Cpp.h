// H5Cpp.h -- no-op stand-in for the HDF5 C++ API.
//
// TEST INFRASTRUCTURE (reference build for the CPU oracle).  The reference's
// Estimator.cpp and simulator.h include H5Cpp.h only for the output.h5
// writer, which the oracle harness never calls.  HDF5 is not installed in this
// image, so these empty types let the reference's own sources compile.
#ifndef ORC_H5CPP_STUB_H
#define ORC_H5CPP_STUB_H
#include <cstddef>
#include <string>

typedef unsigned long long hsize_t;
typedef std::string H5std_string;
#define H5T_VARIABLE ((size_t)-1)
#define H5S_SCALAR 0
#define H5F_ACC_TRUNC 0

namespace H5 {
struct DataType { DataType() {} };
struct PredType : DataType {
    static const DataType NATIVE_DOUBLE;
    static const DataType NATIVE_ULLONG;
};
struct StrType : DataType { StrType(int, size_t) {} };
struct DataSpace {
    DataSpace() {}
    explicit DataSpace(int) {}
    DataSpace(int, const hsize_t *) {}
};
struct Attribute {
    void write(const DataType &, const std::string &) {}
};
struct DataSet {
    void write(const void *, const DataType &) {}
    void write(const std::string &, const DataType &) {}
    Attribute createAttribute(const std::string &, const DataType &, const DataSpace &) { return Attribute(); }
};
struct Group {
    Group createGroup(const std::string &) { return Group(); }
    DataSet createDataSet(const std::string &, const DataType &, const DataSpace &) { return DataSet(); }
    Attribute createAttribute(const std::string &, const DataType &, const DataSpace &) { return Attribute(); }
};
struct H5File : Group {
    H5File() {}
    H5File(const std::string &, int) {}
};
}  // namespace H5
#endif
