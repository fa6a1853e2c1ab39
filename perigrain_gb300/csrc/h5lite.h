// h5lite: a small HDF5 reader/writer covering the subset of the HDF5 file format that
// perigrain's setup input (`data/hdf5/all.h5`, written by h5py) and its per-timestep output
// (`output/hdf5/{tc,wall}_%05u.h5`, `plotinfo.h5`, `run_time.h5`) use.
//
// Written from the public "HDF5 File Format Specification" (version 0 superblock, version 1
// object headers, v1 B-trees with symbol-table nodes and local heaps, contiguous/compact
// layouts, fixed-point and IEEE floating-point datatypes). The reader additionally accepts
// version 2/3 superblocks, version 2 object headers and compact link storage.
//
// Writer output: superblock v0, old-style groups (symbol tables), object header v1, dataspace
// v1, datatype v1, layout v3 contiguous -- the same structures libhdf5 1.8+/h5py produce by
// default, so the files read back with h5py/libhdf5.
#pragma once
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace h5l {

enum class DType : int { F64 = 0, F32 = 1, U32 = 2, I32 = 3, U64 = 4, I64 = 5, U8 = 6 };

size_t dtype_size(DType t);

// ---------------------------------------------------------------------------------------------
// Writer: collect datasets (paths create intermediate groups), then serialize in one pass.
// ---------------------------------------------------------------------------------------------
class Writer {
 public:
  Writer();
  ~Writer();
  // Create an (empty) group; datasets below it create it implicitly as well.
  void create_group(const std::string& path);
  // Add a dataset. `data` holds prod(dims) elements of type `t`, C order. Returns false on a
  // duplicate name or a path that passes through an existing dataset.
  bool add_dataset(const std::string& path, DType t, const std::vector<uint64_t>& dims,
                   const void* data);
  // The same without a copy: `data` must stay valid and unchanged until write()/serialize().
  bool add_dataset_ref(const std::string& path, DType t, const std::vector<uint64_t>& dims,
                       const void* data);
  // Serialize and write the file (truncating). Returns false on I/O error.
  bool write(const std::string& filename) const;
  std::vector<uint8_t> serialize() const;

  struct Node;

 private:
  std::unique_ptr<Node> root_;
  Node* make_group(const std::string& path);
  bool add(const std::string& path, DType t, const std::vector<uint64_t>& dims, const void* data, bool copy);
};

// ---------------------------------------------------------------------------------------------
// Reader
// ---------------------------------------------------------------------------------------------
struct DatasetInfo {
  std::vector<uint64_t> dims;  // empty for a scalar dataspace
  int type_class = -1;         // 0 fixed point, 1 floating point
  uint32_t type_size = 0;
  bool is_signed = false;
  bool big_endian = false;
  uint64_t data_addr = ~0ull;  // contiguous address (or offset of compact data in the header)
  uint64_t data_size = 0;
  bool compact = false;
  std::vector<uint8_t> compact_data;
  uint64_t nelem() const;
};

class Reader {
 public:
  Reader();
  ~Reader();
  // Open and parse the superblock. Returns false (and sets error()) on failure.
  bool open(const std::string& filename);
  bool open_memory(std::vector<uint8_t> bytes);
  const std::string& error() const { return err_; }

  // Look up a dataset by '/'-separated path. Returns false if missing or unsupported.
  bool info(const std::string& path, DatasetInfo* out);
  // Read a dataset converted to `want` (libhdf5-style conversion: integer overflow clamps,
  // float->integer truncates toward zero). dims receives the dataspace extents.
  bool read(const std::string& path, DType want, std::vector<uint64_t>* dims,
            std::vector<uint8_t>* out);
  template <class T>
  bool read_vec(const std::string& path, DType want, std::vector<uint64_t>* dims,
                std::vector<T>* out) {
    std::vector<uint8_t> raw;
    if (!read(path, want, dims, &raw)) return false;
    out->resize(raw.size() / sizeof(T));
    if (!raw.empty()) std::copy(raw.data(), raw.data() + raw.size(), (uint8_t*)out->data());
    return true;
  }
  // Names of the members of a group ("" or "/" for the root), sorted.
  bool list(const std::string& path, std::vector<std::string>* names);
  bool exists(const std::string& path);

 private:
  struct Impl;
  std::unique_ptr<Impl> impl_;
  std::string err_;
};

}  // namespace h5l
