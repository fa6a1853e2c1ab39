// Test infrastructure (oracle): a minimal stand-in for the HDF5 C++ API subset used by the
// reference's src/read/rw_hdf5.h and src/particle/timeloop.h (H5File, DataSet, DataSpace,
// PredType NATIVE_DOUBLE/INT/UINT, createGroup/createDataSet/openDataSet, read/write).
// Backed by the project's HDF5-subset library (perigrain_gb300/csrc/h5lite.*), so the files
// the reference writes through it are real HDF5 files.
#ifndef PERIGRAIN_ORACLE_H5CPP_SHIM
#define PERIGRAIN_ORACLE_H5CPP_SHIM
#include <memory>
#include <string>
#include <typeinfo>
#include <vector>

typedef unsigned long long hsize_t;
#define H5F_ACC_RDONLY 0u
#define H5F_ACC_TRUNC 2u

namespace H5 {

struct FileState;

class PredType {
 public:
  int code;  // h5lite dtype: 0 f64, 2 u32, 3 i32
  explicit PredType(int c) : code(c) {}
  static const PredType NATIVE_DOUBLE;
  static const PredType NATIVE_INT;
  static const PredType NATIVE_UINT;
};

class DataSpace {
 public:
  std::vector<hsize_t> dims;
  DataSpace() {}
  DataSpace(int rank, const hsize_t* d) : dims(d, d + rank) {}
  int getSimpleExtentDims(hsize_t* d, hsize_t* maxdims = nullptr) const;
};

class Group {};

class DataSet {
 public:
  std::shared_ptr<FileState> st;
  std::string path;
  int filetype = 0;
  DataSpace space;
  void write(const void* buf, const PredType& mem) const;
  void read(void* buf, const PredType& mem, const DataSpace& = DataSpace()) const;
  DataSpace getSpace() const { return space; }
};

class H5File {
 public:
  std::shared_ptr<FileState> st;
  H5File(const std::string& name, unsigned flags);
  H5File(const char* name, unsigned flags) : H5File(std::string(name), flags) {}
  void close();
  Group createGroup(const std::string& path);
  DataSet createDataSet(const std::string& path, const PredType& t, const DataSpace& sp);
  DataSet openDataSet(const std::string& path);
};

}  // namespace H5
#endif
