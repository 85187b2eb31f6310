// HDF5 final-state files of the layout the reference writes through libhdf5 (SimIO.hpp;
// outputHDF5Frame with id -1, OutputWriter.cpp:388-441, 736-745: `<name>.Last.h5` holding the
// datasets R, Vel, SigmaCore, F, FD, FR, RHO, Theta, PR, State, T0 and CpuTime in its root
// group), read and written without libhdf5.
//
// The subset is what libhdf5's default file creation makes of such a file: superblock version 0
// or 1, symbol-table groups (version 1 B-trees of any depth, local heap, symbol nodes), version 1
// object headers with continuation blocks, dataspace messages version 1 and 2, little-endian
// fixed-point and IEEE floating-point element types of 1 to 8 bytes, and contiguous or compact
// data (layout messages version 1 to 3). Anything else (chunked or filtered data, version 2
// object headers, big-endian types) is refused with a message, never guessed at.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace cil {
namespace h5 {

struct Dataset {
  std::vector<uint64_t> dims;
  int cls = 0;         // 0 fixed-point, 1 floating-point
  int size = 0;        // bytes per element
  bool is_signed = true;
  bool allocated = true;   // false: never written (reads as zeros, libhdf5's default fill)
  uint64_t addr = 0;       // contiguous data (file offset)
  std::vector<uint8_t> compact;
  bool is_compact = false;
  uint64_t count() const {
    uint64_t n = 1;
    for (uint64_t d : dims) n *= d;
    return n;
  }
};

class Reader {
 public:
  // Reads the whole file; false with *err set when it is not a file of the subset above.
  bool open(const std::string &path, std::string *err);
  // `name`: groups and a dataset from the root ("R", "/snapshots/t_3/R").
  bool dataset(const std::string &name, Dataset *out, std::string *err) const;
  // Any supported element type converted to double (as libhdf5 converts on read).
  bool read(const Dataset &ds, std::vector<double> *out, std::string *err) const;
  // Names in a group ("" or "/" for the root) in the group's name order.
  bool list(const std::string &group, std::vector<std::string> *names, std::string *err) const;
  // A numeric attribute of an object (group or dataset), converted to double.
  bool attribute(const std::string &object, const std::string &name, std::vector<double> *out,
                 std::string *err) const;

 private:
  struct Msg {
    uint16_t type;
    uint64_t off;   // message data offset in the file
    uint16_t size;
  };
  bool messages(uint64_t ohdr, std::vector<Msg> *out, std::string *err) const;
  bool lookup(const std::string &path, uint64_t *ohdr, std::string *err) const;
  bool group_entries(uint64_t ohdr, std::vector<std::pair<std::string, uint64_t>> *out, std::string *err) const;
  bool btree(uint64_t addr, uint64_t heap_data, uint64_t heap_size, int depth,
             std::vector<std::pair<std::string, uint64_t>> *out, std::string *err) const;
  bool in(uint64_t off, uint64_t len) const { return off <= buf_.size() && len <= buf_.size() - off; }
  uint64_t u(uint64_t off, int bytes) const;
  std::vector<uint8_t> buf_;
  uint64_t root_ = 0;
  std::string path_;
};

// Writes a final-state file of the same layout: the datasets in the root group (symbol table:
// one B-tree node of K 16 over symbol nodes of 8 entries, names in a local heap), each with a
// version 1 dataspace (maximum dimensions equal to the dimensions), its element type, a version 2
// fill-value message (late allocation, no fill value) and a version 3 contiguous layout, the
// messages and order of the reference's own files; data stored as FP32 (the reference's
// type_out for double, SimIO.hpp:73) or int32.
class Writer {
 public:
  bool write_f32(const std::string &name, const std::vector<uint64_t> &dims, const double *data, std::string *err);
  bool write_i32(const std::string &name, const std::vector<uint64_t> &dims, const int32_t *data, std::string *err);
  bool save(const std::string &path, std::string *err) const;

 private:
  struct Item {
    std::string name;
    std::vector<uint64_t> dims;
    int cls;
    std::vector<uint8_t> data;
  };
  std::vector<Item> items_;
};

// Writes a frame file of the reference's layout (initHDF5Output / outputHDF5Frame,
// OutputWriter.cpp:240-330, 388-441: /params with the run's attributes, /snapshots/t_<frame>
// with the frame's datasets and its step as the attribute ts) incrementally: each dataset's
// data is appended as it comes, and the metadata (groups as symbol tables, dataset headers as
// Writer lays them out, one-dimensional numeric attributes as in H5LT's set_attribute) is written
// at close, with the superblock. The reference's groups also track the creation order of their
// links; these do not, which readers (h5py, libhdf5) only see when asked for that order.
class FrameFile {
 public:
  bool create(const std::string &path, std::string *err);
  // groups are paths from the root ("params", "snapshots/t_3"), created on first use
  void make_group(const std::string &group);
  bool attr_f64(const std::string &group, const std::string &name, const std::vector<double> &v, std::string *err);
  bool attr_i32(const std::string &group, const std::string &name, const std::vector<int32_t> &v, std::string *err);
  bool data_f32(const std::string &group, const std::string &name, const std::vector<uint64_t> &dims,
                const double *data, std::string *err);
  bool data_i32(const std::string &group, const std::string &name, const std::vector<uint64_t> &dims,
                const int32_t *data, std::string *err);
  bool close(std::string *err);
  ~FrameFile();

 private:
  struct Impl;
  Impl *impl_ = nullptr;
};

}  // namespace h5
}  // namespace cil
