// HDF5 C++ API subset over the project's table container (.mctab).
//
// TEST INFRASTRUCTURE ONLY: lets the reference's HDF5DataSet
// (src/HDF5DataSet.hpp:87-130) read the same tables the engine reads.  A
// pandas DataFrame written by to_hdf stores /pandas/axis1_nlevels, the
// MultiIndex levels /pandas/axis1_level{i} and /pandas/block0_values; the
// container holds exactly those: the level axes and the flattened values.
#pragma once

#include <cstdint>
#include <cstring>
#include <fstream>
#include <iterator>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#define H5F_ACC_RDONLY 0u

namespace H5 {

struct PredType {
  int id;
  static const PredType NATIVE_ULLONG;
  static const PredType NATIVE_DOUBLE;
};
inline const PredType PredType::NATIVE_ULLONG{1};
inline const PredType PredType::NATIVE_DOUBLE{2};

struct Table {
  std::vector<std::vector<double>> axes;
  std::vector<double> values;
};

inline std::shared_ptr<Table> read_table(const std::string& path) {
  std::ifstream in(path, std::ios::binary);
  if (!in) throw std::runtime_error("cannot open " + path);
  std::vector<char> buf((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
  size_t off = 0;
  auto take = [&](void* dst, size_t n) {
    if (off + n > buf.size()) throw std::runtime_error(path + ": truncated table");
    std::memcpy(dst, buf.data() + off, n);
    off += n;
  };
  char magic[8];
  take(magic, 8);
  if (std::memcmp(magic, "MCTAB1\0\0", 8) != 0) throw std::runtime_error(path + ": not a table file");
  uint64_t levels = 0;
  take(&levels, 8);
  auto t = std::make_shared<Table>();
  for (uint64_t i = 0; i < levels; i++) {
    uint64_t n = 0;
    take(&n, 8);
    std::vector<double> a(n);
    take(a.data(), n * 8);
    t->axes.push_back(std::move(a));
  }
  uint64_t nv = 0;
  take(&nv, 8);
  t->values.resize(nv);
  take(t->values.data(), nv * 8);
  return t;
}

class DataSpace {
 public:
  explicit DataSpace(size_t n) : n_(n) {}
  long long getSimpleExtentNpoints() const { return static_cast<long long>(n_); }

 private:
  size_t n_;
};

class DataSet {
 public:
  explicit DataSet(const std::vector<double>* v) : v_(v) {}
  DataSpace getSpace() const { return DataSpace(v_->size()); }
  void read(void* dst, const PredType&) const { std::memcpy(dst, v_->data(), v_->size() * sizeof(double)); }

 private:
  const std::vector<double>* v_;
};

class Attribute {
 public:
  explicit Attribute(unsigned long long v) : v_(v) {}
  void read(const PredType&, void* dst) const { std::memcpy(dst, &v_, sizeof v_); }

 private:
  unsigned long long v_;
};

class Group {
 public:
  explicit Group(std::shared_ptr<Table> t) : t_(std::move(t)) {}
  Attribute openAttribute(const std::string& name) const {
    if (name != "axis1_nlevels") throw std::runtime_error("unknown attribute " + name);
    return Attribute(t_->axes.size());
  }
  DataSet openDataSet(const std::string& name) const {
    if (name == "block0_values") return DataSet(&t_->values);
    const std::string prefix = "axis1_level";
    if (name.compare(0, prefix.size(), prefix) == 0) {
      const size_t i = std::stoul(name.substr(prefix.size()));
      if (i < t_->axes.size()) return DataSet(&t_->axes[i]);
    }
    throw std::runtime_error("unknown data set " + name);
  }

 private:
  std::shared_ptr<Table> t_;
};

class H5File {
 public:
  H5File(const std::string& path, unsigned) : t_(read_table(path)) {}
  Group openGroup(const std::string&) const { return Group(t_); }

 private:
  std::shared_ptr<Table> t_;
};

}  // namespace H5
