// Oracle compat shim (test infrastructure): HighFive/HDF5 are not available, so
// genetIC's gadgethdf/swift writers (genetIC/src/io/gadgethdf.hpp, io/swift.hpp)
// compile against these stand-ins and fail at run time if selected.  They are
// not on the field-realisation path.
#pragma once
#include <stdexcept>
#include <string>
#include <vector>
#include <cstddef>

namespace HighFive {
  struct Exception : std::runtime_error {
    explicit Exception(const std::string &s) : std::runtime_error(s) {}
  };
  [[noreturn]] inline void unavailable() {
    throw Exception("HDF5 output is not available in this build of the reference");
  }
  struct SilenceHDF5 { SilenceHDF5() {} };
  struct DataSpace {
    enum class DataspaceType { dataspace_scalar, dataspace_null };
    DataSpace(size_t) {}
    DataSpace(size_t, size_t) {}
    DataSpace(DataspaceType) {}
  };
  struct Attribute {
    template <typename T> void write(const T &) { unavailable(); }
  };
  struct DataSet {
    template <typename T> void write_raw(const T *) { unavailable(); }
    template <typename T> void write(const T &) { unavailable(); }
  };
  struct Group {
    template <typename T> DataSet createDataSet(const std::string &, const DataSpace &) { unavailable(); }
    template <typename T> Attribute createAttribute(const std::string &, const DataSpace &) { unavailable(); }
  };
  struct File {
    enum : unsigned { ReadOnly = 0, ReadWrite = 1, Truncate = 2, Create = 4 };
    File(const std::string &, unsigned) { unavailable(); }
    Group getGroup(const std::string &) { unavailable(); }
    Group createGroup(const std::string &) { unavailable(); }
  };
}
