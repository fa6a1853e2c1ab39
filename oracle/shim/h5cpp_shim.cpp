// Test infrastructure (oracle): implementation of the H5Cpp.h stand-in over h5lite.
#include "H5Cpp.h"

#include <sys/stat.h>

#include <cstring>
#include <map>
#include <mutex>
#include <stdexcept>

#include "../../perigrain_gb300/csrc/h5lite.h"

namespace H5 {

const PredType PredType::NATIVE_DOUBLE(0);
const PredType PredType::NATIVE_INT(3);
const PredType PredType::NATIVE_UINT(2);

struct FileState {
  std::string name;
  bool writing = false;
  bool closed = false;
  std::mutex mu;
  h5l::Writer w;
  std::shared_ptr<h5l::Reader> r;
  void flush() {
    std::lock_guard<std::mutex> g(mu);
    if (writing && !closed) {
      if (!w.write(name)) throw std::runtime_error("H5 shim: cannot write " + name);
    }
    closed = true;
  }
  ~FileState() {
    try {
      flush();
    } catch (...) {
    }
  }
};

// Readers are cached per (name, size, mtime): the reference re-opens all.h5 once per dataset.
static std::shared_ptr<h5l::Reader> open_reader(const std::string& name) {
  static std::mutex mu;
  static std::map<std::string, std::pair<std::string, std::shared_ptr<h5l::Reader>>> cache;
  struct stat st;
  if (stat(name.c_str(), &st) != 0) throw std::runtime_error("H5 shim: cannot open " + name);
  std::string stamp = std::to_string((long long)st.st_size) + ":" + std::to_string((long long)st.st_mtime) + ":" +
                      std::to_string((long long)st.st_mtim.tv_nsec);
  std::lock_guard<std::mutex> g(mu);
  auto it = cache.find(name);
  if (it != cache.end() && it->second.first == stamp) return it->second.second;
  auto r = std::make_shared<h5l::Reader>();
  if (!r->open(name)) throw std::runtime_error("H5 shim: " + name + ": " + r->error());
  cache[name] = {stamp, r};
  return r;
}

int DataSpace::getSimpleExtentDims(hsize_t* d, hsize_t* maxdims) const {
  for (size_t i = 0; i < dims.size(); ++i) {
    d[i] = dims[i];
    if (maxdims) maxdims[i] = dims[i];
  }
  return (int)dims.size();
}

H5File::H5File(const std::string& name, unsigned flags) : st(std::make_shared<FileState>()) {
  st->name = name;
  if (flags == H5F_ACC_TRUNC) {
    st->writing = true;
  } else {
    st->r = open_reader(name);
  }
}

void H5File::close() { st->flush(); }

Group H5File::createGroup(const std::string& path) {
  std::lock_guard<std::mutex> g(st->mu);
  st->w.create_group(path);
  return Group();
}

DataSet H5File::createDataSet(const std::string& path, const PredType& t, const DataSpace& sp) {
  DataSet d;
  d.st = st;
  d.path = path;
  d.filetype = t.code;
  d.space = sp;
  return d;
}

DataSet H5File::openDataSet(const std::string& path) {
  h5l::DatasetInfo info;
  if (!st->r || !st->r->info(path, &info))
    throw std::runtime_error("H5 shim: " + st->name + ": cannot open dataset " + path);
  DataSet d;
  d.st = st;
  d.path = path;
  d.space.dims.assign(info.dims.begin(), info.dims.end());
  return d;
}

void DataSet::write(const void* buf, const PredType& mem) const {
  if (mem.code != filetype) throw std::runtime_error("H5 shim: type conversion on write is not supported");
  std::lock_guard<std::mutex> g(st->mu);
  std::vector<uint64_t> dims(space.dims.begin(), space.dims.end());
  if (!st->w.add_dataset(path, (h5l::DType)filetype, dims, buf))
    throw std::runtime_error("H5 shim: cannot create dataset " + path);
}

void DataSet::read(void* buf, const PredType& mem, const DataSpace&) const {
  std::vector<uint64_t> dims;
  std::vector<uint8_t> raw;
  if (!st->r->read(path, (h5l::DType)mem.code, &dims, &raw))
    throw std::runtime_error("H5 shim: cannot read " + path + ": " + st->r->error());
  if (!raw.empty()) std::memcpy(buf, raw.data(), raw.size());
}

}  // namespace H5
