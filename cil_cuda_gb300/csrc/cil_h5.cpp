// HDF5 final-state files without libhdf5 (cil_h5.hpp). Field layouts follow the published HDF5
// file format specification (superblock version 0/1, version 1 B-trees of group nodes, local
// heaps, symbol table nodes, version 1 object headers and their messages).
#include "cil_h5.hpp"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <functional>
#include <iterator>
#include <limits>

#include "cil_input.h"

namespace cil {
namespace h5 {

namespace {

constexpr uint64_t kUndef = std::numeric_limits<uint64_t>::max();
const uint8_t kSig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};

// message types
constexpr uint16_t kDataspace = 0x01, kDatatype = 0x03, kFillNew = 0x05, kLayout = 0x08, kFilters = 0x0B,
                   kCont = 0x10, kSymtab = 0x11;

bool fail(std::string *err, const std::string &m) {
  if (err) *err = m;
  return false;
}

}  // namespace

uint64_t Reader::u(uint64_t off, int bytes) const {
  uint64_t v = 0;
  for (int k = bytes - 1; k >= 0; --k) v = (v << 8) | buf_[off + k];
  return v;
}

bool Reader::open(const std::string &path, std::string *err) {
  path_ = path;
  std::ifstream f(path, std::ios::binary);
  if (!f) return fail(err, path + ": cannot open");
  buf_.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
  // the superblock is at 0 or at the first power of two >= 512 holding the signature
  uint64_t sb = 0;
  for (uint64_t at = 0; at + 8 <= buf_.size(); at = at == 0 ? 512 : at * 2) {
    if (std::memcmp(buf_.data() + at, kSig, 8) == 0) {
      sb = at;
      break;
    }
    if (at >= (uint64_t(1) << 40)) return fail(err, path + ": not an HDF5 file");
  }
  if (!in(sb, 8) || std::memcmp(buf_.data() + sb, kSig, 8) != 0) return fail(err, path + ": not an HDF5 file");
  if (!in(sb, 24)) return fail(err, path + ": truncated superblock");
  const int ver = buf_[sb + 8];
  if (ver != 0 && ver != 1)
    return fail(err, path + ": superblock version " + std::to_string(ver) + " (only 0 and 1, libhdf5's default, are read)");
  if (buf_[sb + 13] != 8 || buf_[sb + 14] != 8) return fail(err, path + ": offsets and lengths other than 8 bytes");
  // version 1 adds the indexed-storage K and 2 reserved bytes
  const uint64_t base = sb + 24 + (ver == 1 ? 4 : 0);
  const uint64_t entry = base + 32;  // after base, free-space, end-of-file and driver addresses
  if (!in(entry, 40)) return fail(err, path + ": truncated superblock");
  root_ = u(entry + 8, 8);
  if (!in(root_, 16)) return fail(err, path + ": root object header outside the file");
  return true;
}

bool Reader::messages(uint64_t ohdr, std::vector<Msg> *out, std::string *err) const {
  out->clear();
  if (!in(ohdr, 16)) return fail(err, "object header outside the file");
  if (buf_[ohdr] != 1) {
    if (in(ohdr, 4) && std::memcmp(buf_.data() + ohdr, "OHDR", 4) == 0)
      return fail(err, "version 2 object headers are not read");
    return fail(err, "object header version " + std::to_string(buf_[ohdr]));
  }
  const uint64_t nmsg = u(ohdr + 2, 2);
  std::vector<std::pair<uint64_t, uint64_t>> blocks{{ohdr + 16, u(ohdr + 8, 4)}};
  for (size_t b = 0; b < blocks.size() && out->size() < nmsg; ++b) {
    uint64_t p = blocks[b].first;
    if (!in(p, blocks[b].second)) return fail(err, "object header block outside the file");
    const uint64_t end = p + blocks[b].second;
    while (p + 8 <= end && out->size() < nmsg) {
      Msg m{static_cast<uint16_t>(u(p, 2)), p + 8, static_cast<uint16_t>(u(p + 2, 2))};
      if (m.off + m.size > end) return fail(err, "object header message overruns its block");
      if (m.type == kCont) {
        if (m.size < 16) return fail(err, "short continuation message");
        blocks.push_back({u(m.off, 8), u(m.off + 8, 8)});
        if (blocks.size() > 4096) return fail(err, "too many object header continuations");
      }
      out->push_back(m);
      p = m.off + m.size;
    }
  }
  return true;
}

bool Reader::btree(uint64_t addr, uint64_t heap_data, uint64_t heap_size, int depth,
                   std::vector<std::pair<std::string, uint64_t>> *out, std::string *err) const {
  if (depth > 64) return fail(err, "B-tree deeper than 64 levels");
  if (!in(addr, 24) || std::memcmp(buf_.data() + addr, "TREE", 4) != 0) return fail(err, "bad group B-tree node");
  if (buf_[addr + 4] != 0) return fail(err, "B-tree node of a raw-data index in a group");
  const int level = buf_[addr + 5];
  const uint64_t used = u(addr + 6, 2);
  if (!in(addr + 24, (2 * used + 1) * 8)) return fail(err, "B-tree node outside the file");
  for (uint64_t k = 0; k < used; ++k) {
    const uint64_t child = u(addr + 24 + (2 * k + 1) * 8, 8);
    if (level > 0) {
      if (!btree(child, heap_data, heap_size, depth + 1, out, err)) return false;
      continue;
    }
    if (!in(child, 8) || std::memcmp(buf_.data() + child, "SNOD", 4) != 0) return fail(err, "bad symbol table node");
    const uint64_t n = u(child + 6, 2);
    if (!in(child + 8, n * 40)) return fail(err, "symbol table node outside the file");
    for (uint64_t e = 0; e < n; ++e) {
      const uint64_t q = child + 8 + e * 40;
      const uint64_t name_off = u(q, 8);
      if (name_off >= heap_size) return fail(err, "link name outside the local heap");
      const char *s = reinterpret_cast<const char *>(buf_.data() + heap_data + name_off);
      const size_t len = strnlen(s, heap_size - name_off);
      out->push_back({std::string(s, len), u(q + 8, 8)});
    }
  }
  return true;
}

bool Reader::group_entries(uint64_t ohdr, std::vector<std::pair<std::string, uint64_t>> *out,
                           std::string *err) const {
  std::vector<Msg> ms;
  if (!messages(ohdr, &ms, err)) return false;
  for (const Msg &m : ms) {
    if (m.type != kSymtab) continue;
    if (m.size < 16) return fail(err, "short symbol table message");
    const uint64_t tree = u(m.off, 8), heap = u(m.off + 8, 8);
    if (!in(heap, 32) || std::memcmp(buf_.data() + heap, "HEAP", 4) != 0) return fail(err, "bad local heap");
    const uint64_t hsize = u(heap + 8, 8), hdata = u(heap + 24, 8);
    if (!in(hdata, hsize)) return fail(err, "local heap data outside the file");
    out->clear();
    return btree(tree, hdata, hsize, 0, out, err);
  }
  return fail(err, "not a group of symbol-table form (link messages are not read)");
}

bool Reader::lookup(const std::string &path, uint64_t *ohdr, std::string *err) const {
  uint64_t cur = root_;
  size_t p = 0;
  while (p < path.size()) {
    while (p < path.size() && path[p] == '/') ++p;
    if (p >= path.size()) break;
    size_t q = path.find('/', p);
    if (q == std::string::npos) q = path.size();
    const std::string part = path.substr(p, q - p);
    std::vector<std::pair<std::string, uint64_t>> es;
    if (!group_entries(cur, &es, err)) return fail(err, path_ + ": " + path + ": " + *err);
    auto it = std::find_if(es.begin(), es.end(), [&](const auto &e) { return e.first == part; });
    if (it == es.end()) return fail(err, path_ + ": no object " + path);
    cur = it->second;
    p = q;
  }
  *ohdr = cur;
  return true;
}

bool Reader::list(const std::string &group, std::vector<std::string> *names, std::string *err) const {
  uint64_t oh;
  if (!lookup(group, &oh, err)) return false;
  std::vector<std::pair<std::string, uint64_t>> es;
  if (!group_entries(oh, &es, err)) return false;
  names->clear();
  for (const auto &e : es) names->push_back(e.first);
  return true;
}

bool Reader::dataset(const std::string &name, Dataset *out, std::string *err) const {
  uint64_t oh;
  if (!lookup(name, &oh, err)) return false;
  std::vector<Msg> ms;
  if (!messages(oh, &ms, err)) return fail(err, path_ + ": " + name + ": " + *err);
  const std::string where = path_ + ": " + name + ": ";
  *out = Dataset{};
  bool have_space = false, have_type = false, have_layout = false;
  for (const Msg &m : ms) {
    const uint64_t d = m.off;
    if (m.type == kDataspace) {
      if (m.size < 8) return fail(err, where + "short dataspace message");
      const int ver = buf_[d], rank = buf_[d + 1];
      const uint64_t dims_at = ver == 1 ? d + 8 : d + 4;
      if (ver != 1 && ver != 2) return fail(err, where + "dataspace message version " + std::to_string(ver));
      if (ver == 2 && buf_[d + 3] == 2) return fail(err, where + "null dataspace");
      if (dims_at + 8 * static_cast<uint64_t>(rank) > d + m.size) return fail(err, where + "short dataspace message");
      for (int k = 0; k < rank; ++k) out->dims.push_back(u(dims_at + 8 * k, 8));
      have_space = true;
    } else if (m.type == kDatatype) {
      if (m.size < 8) return fail(err, where + "short datatype message");
      const int cls = buf_[d] & 0x0f;
      const uint8_t bits0 = buf_[d + 1];
      out->size = static_cast<int>(u(d + 4, 4));
      if (cls != 0 && cls != 1) return fail(err, where + "element class " + std::to_string(cls) + " (numbers only)");
      if (bits0 & 0x01) return fail(err, where + "big-endian elements");
      if (cls == 0 && out->size != 1 && out->size != 2 && out->size != 4 && out->size != 8)
        return fail(err, where + "integer of " + std::to_string(out->size) + " bytes");
      if (cls == 1 && out->size != 4 && out->size != 8)
        return fail(err, where + "floating point of " + std::to_string(out->size) + " bytes");
      out->cls = cls;
      out->is_signed = cls == 1 || (bits0 & 0x08) != 0;
      have_type = true;
    } else if (m.type == kLayout) {
      const int ver = buf_[d];
      if (ver == 3) {
        const int lc = buf_[d + 1];
        if (lc == 0) {
          const uint64_t sz = u(d + 2, 2);
          if (4 + sz > m.size) return fail(err, where + "short compact layout");
          out->is_compact = true;
          out->compact.assign(buf_.begin() + d + 4, buf_.begin() + d + 4 + sz);
        } else if (lc == 1) {
          out->addr = u(d + 2, 8);
          out->allocated = out->addr != kUndef;
        } else {
          return fail(err, where + "chunked or virtual data (contiguous and compact only)");
        }
      } else if (ver == 1 || ver == 2) {
        const int ndims = buf_[d + 1], lc = buf_[d + 2];
        if (lc == 1) {
          out->addr = u(d + 8, 8);
          out->allocated = out->addr != kUndef;
        } else if (lc == 0) {
          const uint64_t at = d + 8 + 4 * static_cast<uint64_t>(ndims);
          const uint64_t sz = u(at, 4);
          out->is_compact = true;
          out->compact.assign(buf_.begin() + at + 4, buf_.begin() + at + 4 + sz);
        } else {
          return fail(err, where + "chunked data (contiguous and compact only)");
        }
      } else {
        return fail(err, where + "layout message version " + std::to_string(ver));
      }
      have_layout = true;
    } else if (m.type == kFilters) {
      return fail(err, where + "filtered (compressed) data");
    }
  }
  if (!have_space || !have_type || !have_layout) return fail(err, where + "not a dataset");
  const uint64_t bytes = out->count() * static_cast<uint64_t>(out->size);
  if (out->is_compact ? out->compact.size() < bytes : (out->allocated && !in(out->addr, bytes)))
    return fail(err, where + "data outside the file");
  return true;
}

bool Reader::read(const Dataset &ds, std::vector<double> *out, std::string *err) const {
  const uint64_t n = ds.count();
  out->assign(n, 0.0);
  if (!ds.allocated) return true;
  const uint8_t *p = ds.is_compact ? ds.compact.data() : buf_.data() + ds.addr;
  for (uint64_t i = 0; i < n; ++i) {
    const uint8_t *q = p + i * ds.size;
    uint64_t v = 0;
    for (int k = ds.size - 1; k >= 0; --k) v = (v << 8) | q[k];
    double x;
    if (ds.cls == 1) {
      if (ds.size == 4) {
        const uint32_t w = static_cast<uint32_t>(v);
        float f;
        std::memcpy(&f, &w, 4);
        x = f;
      } else {
        std::memcpy(&x, &v, 8);
      }
    } else if (ds.is_signed) {
      const int sh = 64 - 8 * ds.size;
      x = static_cast<double>(static_cast<int64_t>(v << sh) >> sh);
    } else {
      x = static_cast<double>(v);
    }
    (*out)[i] = x;
  }
  (void)err;
  return true;
}

bool Reader::attribute(const std::string &object, const std::string &name, std::vector<double> *out,
                       std::string *err) const {
  uint64_t oh;
  if (!lookup(object, &oh, err)) return false;
  std::vector<Msg> ms;
  if (!messages(oh, &ms, err)) return false;
  const std::string where = path_ + ": " + object + ": attribute " + name + ": ";
  for (const Msg &m : ms) {
    if (m.type != 0x0C || m.size < 8) continue;
    const uint64_t d = m.off;
    if (buf_[d] != 1) continue;  // version 1 (object headers of version 1)
    const uint64_t nsz = u(d + 2, 2), tsz = u(d + 4, 2), ssz = u(d + 6, 2);
    auto pad8 = [](uint64_t x) { return (x + 7) / 8 * 8; };
    const uint64_t at_name = d + 8, at_type = at_name + pad8(nsz), at_space = at_type + pad8(tsz),
                   at_data = at_space + pad8(ssz);
    if (at_data > d + m.size || nsz == 0) return fail(err, where + "malformed attribute message");
    const std::string an(reinterpret_cast<const char *>(buf_.data() + at_name), strnlen(
        reinterpret_cast<const char *>(buf_.data() + at_name), nsz));
    if (an != name) continue;
    const int cls = buf_[at_type] & 0x0f, size = static_cast<int>(u(at_type + 4, 4));
    const bool sgn = cls == 1 || (buf_[at_type + 1] & 0x08);
    if ((cls != 0 && cls != 1) || (buf_[at_type + 1] & 0x01) || (cls == 1 && size != 4 && size != 8) ||
        (cls == 0 && size != 1 && size != 2 && size != 4 && size != 8))
      return fail(err, where + "not a little-endian number");
    const int sver = buf_[at_space], rank = buf_[at_space + 1];
    const uint64_t dims_at = sver == 1 ? at_space + 8 : at_space + 4;
    uint64_t n = 1;
    for (int k = 0; k < rank; ++k) n *= u(dims_at + 8 * k, 8);
    if (at_data + n * size > d + m.size) return fail(err, where + "data outside its message");
    out->assign(n, 0.0);
    for (uint64_t i = 0; i < n; ++i) {
      const uint64_t q = at_data + i * size;
      const uint64_t v = u(q, size);
      double x;
      if (cls == 1) {
        if (size == 4) {
          const uint32_t w = static_cast<uint32_t>(v);
          float fl;
          std::memcpy(&fl, &w, 4);
          x = fl;
        } else {
          std::memcpy(&x, &v, 8);
        }
      } else if (sgn) {
        const int sh = 64 - 8 * size;
        x = static_cast<double>(static_cast<int64_t>(v << sh) >> sh);
      } else {
        x = static_cast<double>(v);
      }
      (*out)[i] = x;
    }
    return true;
  }
  return fail(err, where + "not found");
}

// ---------------------------------------------------------------------------- writer
namespace {

struct Buf {
  std::vector<uint8_t> b;
  void put(uint64_t v, int bytes) {
    for (int k = 0; k < bytes; ++k) b.push_back(static_cast<uint8_t>(v >> (8 * k)));
  }
  void bytes(const void *p, size_t n) {
    const uint8_t *q = static_cast<const uint8_t *>(p);
    b.insert(b.end(), q, q + n);
  }
  void pad8() {
    while (b.size() % 8) b.push_back(0);
  }
  void set(size_t at, uint64_t v, int bytes) {
    for (int k = 0; k < bytes; ++k) b[at + k] = static_cast<uint8_t>(v >> (8 * k));
  }
};

constexpr int kLeafK = 4;       // symbol node: 2K = 8 entries
constexpr int kInternalK = 16;  // group B-tree node: 2K = 32 children

void message(Buf &oh, uint16_t type, uint8_t flags, const Buf &data) {
  Buf d = data;
  d.pad8();
  oh.put(type, 2);
  oh.put(d.b.size(), 2);
  oh.put(flags, 1);
  oh.put(0, 3);
  oh.bytes(d.b.data(), d.b.size());
}

}  // namespace

bool Writer::write_f32(const std::string &name, const std::vector<uint64_t> &dims, const double *data,
                       std::string *err) {
  Item it{name, dims, 1, {}};
  uint64_t n = 1;
  for (uint64_t d : dims) n *= d;
  it.data.resize(n * 4);
  for (uint64_t i = 0; i < n; ++i) {
    const float f = static_cast<float>(data[i]);
    std::memcpy(it.data.data() + 4 * i, &f, 4);
  }
  if (name.empty() || name.find('/') != std::string::npos) return fail(err, "dataset names are plain names");
  items_.push_back(std::move(it));
  return true;
}

bool Writer::write_i32(const std::string &name, const std::vector<uint64_t> &dims, const int32_t *data,
                       std::string *err) {
  Item it{name, dims, 0, {}};
  uint64_t n = 1;
  for (uint64_t d : dims) n *= d;
  it.data.resize(n * 4);
  if (n) std::memcpy(it.data.data(), data, n * 4);
  if (name.empty() || name.find('/') != std::string::npos) return fail(err, "dataset names are plain names");
  items_.push_back(std::move(it));
  return true;
}

bool Writer::save(const std::string &path, std::string *err) const {
  std::vector<const Item *> items;
  for (const Item &it : items_) items.push_back(&it);
  std::sort(items.begin(), items.end(), [](const Item *a, const Item *b) { return a->name < b->name; });
  for (size_t k = 1; k < items.size(); ++k)
    if (items[k]->name == items[k - 1]->name) return fail(err, "dataset " + items[k]->name + " written twice");
  const size_t nsnod = (items.size() + 2 * kLeafK - 1) / (2 * kLeafK);
  if (nsnod > 2 * kInternalK) return fail(err, "more than 256 datasets in one file");

  // local heap data: "" at 0, then the names, each padded to 8 bytes
  Buf heap;
  heap.put(0, 8);
  std::vector<uint64_t> name_off;
  for (const Item *it : items) {
    name_off.push_back(heap.b.size());
    heap.bytes(it->name.c_str(), it->name.size() + 1);
    heap.pad8();
  }
  // addresses: superblock (96), root object header (40), B-tree node, local heap header and
  // data, symbol nodes, dataset object headers, raw data
  const uint64_t a_root = 96, a_tree = a_root + 40;
  const uint64_t tree_size = 24 + (2 * kInternalK + 1) * 8 + 2 * kInternalK * 8;
  const uint64_t a_heap = a_tree + tree_size, a_heap_data = a_heap + 32;
  const uint64_t a_snod = a_heap_data + heap.b.size();
  const uint64_t snod_size = 8 + 2 * kLeafK * 40;
  uint64_t at = a_snod + std::max<size_t>(nsnod, 1) * snod_size;
  std::vector<Buf> ohs;
  std::vector<uint64_t> a_oh;
  for (const Item *it : items) {
    Buf oh;
    Buf sp;  // dataspace v1 with maximum dimensions
    sp.put(1, 1);
    sp.put(it->dims.size(), 1);
    sp.put(1, 1);
    sp.put(0, 5);
    for (uint64_t d : it->dims) sp.put(d, 8);
    for (uint64_t d : it->dims) sp.put(d, 8);
    Buf ty;
    if (it->cls == 1) {  // IEEE binary32 little-endian
      ty.put(0x11, 1);
      ty.put(0x20, 1);
      ty.put(31, 1);
      ty.put(0, 1);
      ty.put(4, 4);
      ty.put(0, 2);
      ty.put(32, 2);
      ty.put(23, 1);
      ty.put(8, 1);
      ty.put(0, 1);
      ty.put(23, 1);
      ty.put(127, 4);
    } else {  // signed 32-bit little-endian
      ty.put(0x10, 1);
      ty.put(0x08, 1);
      ty.put(0, 2);
      ty.put(4, 4);
      ty.put(0, 2);
      ty.put(32, 2);
    }
    Buf fill;  // version 2: late allocation, fill written if set, fill value defined, size 0
    fill.put(2, 1);
    fill.put(2, 1);
    fill.put(2, 1);
    fill.put(1, 1);
    fill.put(0, 4);
    Buf lay;  // version 3 contiguous; address patched below
    lay.put(3, 1);
    lay.put(1, 1);
    lay.put(0, 8);
    lay.put(it->data.size(), 8);
    Buf msgs;
    message(msgs, kDataspace, 0, sp);
    message(msgs, kDatatype, 1, ty);
    message(msgs, kFillNew, 1, fill);
    message(msgs, kLayout, 0, lay);
    oh.put(1, 1);
    oh.put(0, 1);
    oh.put(4, 2);
    oh.put(1, 4);
    oh.put(msgs.b.size(), 4);
    oh.put(0, 4);
    oh.bytes(msgs.b.data(), msgs.b.size());
    a_oh.push_back(at);
    at += oh.b.size();
    ohs.push_back(std::move(oh));
  }
  std::vector<uint64_t> a_data;
  for (size_t k = 0; k < items.size(); ++k) {
    at = (at + 7) / 8 * 8;
    a_data.push_back(at);
    at += items[k]->data.size();
    // the layout message is the last one: its address field sits 18 + 8 bytes before the end
    Buf &oh = ohs[k];
    oh.set(oh.b.size() - 24 + 2, a_data.back(), 8);
  }
  const uint64_t eof = at;

  Buf f;
  f.bytes(kSig, 8);
  f.put(0, 1);  // superblock version
  f.put(0, 1);  // free-space version
  f.put(0, 1);  // root group symbol table version
  f.put(0, 1);
  f.put(0, 1);  // shared header version
  f.put(8, 1);  // sizes of offsets and lengths
  f.put(8, 1);
  f.put(0, 1);
  f.put(kLeafK, 2);
  f.put(kInternalK, 2);
  f.put(0, 4);  // consistency flags
  f.put(0, 8);  // base address
  f.put(kUndef, 8);
  f.put(eof, 8);
  f.put(kUndef, 8);
  // root symbol table entry: name offset, object header, cache type 1 with B-tree and heap
  f.put(0, 8);
  f.put(a_root, 8);
  f.put(1, 4);
  f.put(0, 4);
  f.put(a_tree, 8);
  f.put(a_heap, 8);
  // root object header: one symbol table message
  {
    Buf st;
    st.put(a_tree, 8);
    st.put(a_heap, 8);
    Buf msgs;
    message(msgs, kSymtab, 0, st);
    f.put(1, 1);
    f.put(0, 1);
    f.put(1, 2);
    f.put(1, 4);
    f.put(msgs.b.size(), 4);
    f.put(0, 4);
    f.bytes(msgs.b.data(), msgs.b.size());
  }
  // B-tree node (level 0): key 0 = "" then, after each child, the offset of its last name
  {
    const size_t start = f.b.size();
    f.bytes("TREE", 4);
    f.put(0, 1);
    f.put(0, 1);
    f.put(nsnod, 2);
    f.put(kUndef, 8);
    f.put(kUndef, 8);
    f.put(0, 8);
    for (size_t s = 0; s < nsnod; ++s) {
      const size_t last = std::min(items.size(), (s + 1) * 2 * kLeafK) - 1;
      f.put(a_snod + s * snod_size, 8);
      f.put(name_off[last], 8);
    }
    f.b.resize(start + tree_size, 0);
  }
  // local heap header: no free block (offset 1 marks the empty free list)
  f.bytes("HEAP", 4);
  f.put(0, 4);
  f.put(heap.b.size(), 8);
  f.put(1, 8);
  f.put(a_heap_data, 8);
  f.bytes(heap.b.data(), heap.b.size());
  // symbol nodes
  for (size_t s = 0; s < std::max<size_t>(nsnod, 1); ++s) {
    const size_t start = f.b.size();
    f.bytes("SNOD", 4);
    f.put(1, 1);
    f.put(0, 1);
    const size_t lo = s * 2 * kLeafK, hi = std::min(items.size(), lo + 2 * kLeafK);
    f.put(hi > lo ? hi - lo : 0, 2);
    for (size_t k = lo; k < hi; ++k) {
      f.put(name_off[k], 8);
      f.put(a_oh[k], 8);
      f.put(0, 4);
      f.put(0, 4);
      f.put(0, 16);
    }
    f.b.resize(start + snod_size, 0);
  }
  for (const Buf &oh : ohs) f.bytes(oh.b.data(), oh.b.size());
  for (size_t k = 0; k < items.size(); ++k) {
    f.b.resize(a_data[k], 0);
    f.bytes(items[k]->data.data(), items[k]->data.size());
  }
  if (f.b.size() != eof) return fail(err, "internal layout error");
  std::ofstream o(path, std::ios::binary | std::ios::trunc);
  if (!o) return fail(err, path + ": cannot create");
  o.write(reinterpret_cast<const char *>(f.b.data()), static_cast<std::streamsize>(f.b.size()));
  if (!o) return fail(err, path + ": write failed");
  return true;
}

}  // namespace h5
}  // namespace cil

// ---------------------------------------------------------------------------- frame file
namespace cil {
namespace h5 {
namespace {

Buf space_v1(const std::vector<uint64_t> &dims) {  // dataspace v1, maximum dimensions = dimensions
  Buf sp;
  sp.put(1, 1);
  sp.put(dims.size(), 1);
  sp.put(1, 1);
  sp.put(0, 5);
  for (uint64_t d : dims) sp.put(d, 8);
  for (uint64_t d : dims) sp.put(d, 8);
  return sp;
}

Buf type_of(int cls, int size) {
  Buf ty;
  if (cls == 1 && size == 4) {  // IEEE binary32 little-endian
    ty.put(0x11, 1);
    ty.put(0x20, 1);
    ty.put(31, 1);
    ty.put(0, 1);
    ty.put(4, 4);
    ty.put(0, 2);
    ty.put(32, 2);
    ty.put(23, 1);
    ty.put(8, 1);
    ty.put(0, 1);
    ty.put(23, 1);
    ty.put(127, 4);
  } else if (cls == 1) {  // IEEE binary64 little-endian
    ty.put(0x11, 1);
    ty.put(0x20, 1);
    ty.put(63, 1);
    ty.put(0, 1);
    ty.put(8, 4);
    ty.put(0, 2);
    ty.put(64, 2);
    ty.put(52, 1);
    ty.put(11, 1);
    ty.put(0, 1);
    ty.put(52, 1);
    ty.put(1023, 4);
  } else {  // signed 32-bit little-endian
    ty.put(0x10, 1);
    ty.put(0x08, 1);
    ty.put(0, 2);
    ty.put(4, 4);
    ty.put(0, 2);
    ty.put(32, 2);
  }
  return ty;
}

}  // namespace

struct FrameFile::Impl {
  struct Attr {
    std::string name;
    int cls, size;
    std::vector<uint8_t> bytes;
    uint64_t n;
  };
  struct Data {
    std::string name;
    std::vector<uint64_t> dims;
    int cls;
    uint64_t addr, bytes;
  };
  struct Group {
    std::string name;
    std::vector<Group *> groups;
    std::vector<Data> data;
    std::vector<Attr> attrs;
    uint64_t oh = 0, tree = 0, heap = 0;
    ~Group() {
      for (Group *g : groups) delete g;
    }
  };
  std::string path;
  std::FILE *f = nullptr;
  uint64_t eof = 0;
  Group root;

  Group *group(const std::string &p) {
    Group *g = &root;
    size_t i = 0;
    while (i < p.size()) {
      while (i < p.size() && p[i] == '/') ++i;
      if (i >= p.size()) break;
      size_t j = p.find('/', i);
      if (j == std::string::npos) j = p.size();
      const std::string part = p.substr(i, j - i);
      Group *next = nullptr;
      for (Group *c : g->groups)
        if (c->name == part) next = c;
      if (!next) {
        next = new Group();
        next->name = part;
        g->groups.push_back(next);
      }
      g = next;
      i = j;
    }
    return g;
  }

  bool append(const void *p, size_t n, uint64_t *at, std::string *err) {
    static const uint8_t zeros[8] = {0};
    const uint64_t pad = (8 - eof % 8) % 8;
    if (pad && std::fwrite(zeros, 1, pad, f) != pad) return fail(err, path + ": write failed");
    eof += pad;
    *at = eof;
    if (n && std::fwrite(p, 1, n, f) != n) return fail(err, path + ": write failed");
    eof += n;
    return true;
  }
};

bool FrameFile::create(const std::string &path, std::string *err) {
  delete impl_;
  impl_ = new Impl();
  impl_->path = path;
  impl_->f = std::fopen(path.c_str(), "wb");
  if (!impl_->f) return fail(err, path + ": cannot create");
  // the superblock and the root's entry, written again at close
  static const uint8_t zeros[96] = {0};
  if (std::fwrite(zeros, 1, 96, impl_->f) != 96) return fail(err, path + ": write failed");
  impl_->eof = 96;
  return true;
}

FrameFile::~FrameFile() {
  if (impl_ && impl_->f) std::fclose(impl_->f);
  delete impl_;
}

void FrameFile::make_group(const std::string &group) {
  if (impl_) impl_->group(group);
}

bool FrameFile::attr_f64(const std::string &group, const std::string &name, const std::vector<double> &v,
                         std::string *err) {
  if (!impl_ || !impl_->f) return fail(err, "frame file not open");
  Impl::Attr a{name, 1, 8, std::vector<uint8_t>(v.size() * 8), v.size()};
  if (!v.empty()) std::memcpy(a.bytes.data(), v.data(), v.size() * 8);
  impl_->group(group)->attrs.push_back(std::move(a));
  return true;
}

bool FrameFile::attr_i32(const std::string &group, const std::string &name, const std::vector<int32_t> &v,
                         std::string *err) {
  if (!impl_ || !impl_->f) return fail(err, "frame file not open");
  Impl::Attr a{name, 0, 4, std::vector<uint8_t>(v.size() * 4), v.size()};
  if (!v.empty()) std::memcpy(a.bytes.data(), v.data(), v.size() * 4);
  impl_->group(group)->attrs.push_back(std::move(a));
  return true;
}

bool FrameFile::data_f32(const std::string &group, const std::string &name, const std::vector<uint64_t> &dims,
                         const double *data, std::string *err) {
  if (!impl_ || !impl_->f) return fail(err, "frame file not open");
  uint64_t n = 1;
  for (uint64_t d : dims) n *= d;
  std::vector<float> v(n);
  for (uint64_t i = 0; i < n; ++i) v[i] = static_cast<float>(data[i]);
  uint64_t at;
  if (!impl_->append(v.data(), n * 4, &at, err)) return false;
  impl_->group(group)->data.push_back({name, dims, 1, at, n * 4});
  return true;
}

bool FrameFile::data_i32(const std::string &group, const std::string &name, const std::vector<uint64_t> &dims,
                         const int32_t *data, std::string *err) {
  if (!impl_ || !impl_->f) return fail(err, "frame file not open");
  uint64_t n = 1;
  for (uint64_t d : dims) n *= d;
  uint64_t at;
  if (!impl_->append(data, n * 4, &at, err)) return false;
  impl_->group(group)->data.push_back({name, dims, 0, at, n * 4});
  return true;
}

bool FrameFile::close(std::string *err) {
  if (!impl_ || !impl_->f) return fail(err, "frame file not open");
  Impl &I = *impl_;
  // one B-tree node per group: K large enough for the largest group
  size_t most = 0;
  std::vector<Impl::Group *> all{&I.root};
  for (size_t k = 0; k < all.size(); ++k) {
    most = std::max(most, all[k]->groups.size() + all[k]->data.size());
    for (Impl::Group *c : all[k]->groups) all.push_back(c);
  }
  const size_t most_snod = (most + 2 * kLeafK - 1) / (2 * kLeafK);
  const int K = static_cast<int>(std::max<size_t>(kInternalK, (most_snod + 1) / 2));
  if (K > 65535) return fail(err, "too many entries in one group");
  const uint64_t tree_size = 24 + (2 * static_cast<uint64_t>(K) + 1) * 8 + 2 * static_cast<uint64_t>(K) * 8;
  const uint64_t snod_size = 8 + 2 * kLeafK * 40;
  uint64_t at = (I.eof + 7) / 8 * 8;
  Buf meta;  // written at `base`
  const uint64_t base = at;
  auto here = [&]() { return base + meta.b.size(); };
  // post-order: children first, so that a group's entries know their object headers
  std::function<bool(Impl::Group &)> emit = [&](Impl::Group &g) -> bool {
    struct Entry {
      std::string name;
      uint64_t oh;
      bool group;
      Impl::Group *gp;
    };
    std::vector<Entry> es;
    for (Impl::Group *c : g.groups) {
      if (!emit(*c)) return false;
      es.push_back({c->name, c->oh, true, c});
    }
    for (const Impl::Data &d : g.data) {
      Buf msgs;
      message(msgs, kDataspace, 0, space_v1(d.dims));
      message(msgs, kDatatype, 1, type_of(d.cls, 4));
      Buf fill;
      fill.put(2, 1);
      fill.put(2, 1);
      fill.put(2, 1);
      fill.put(1, 1);
      fill.put(0, 4);
      message(msgs, kFillNew, 1, fill);
      Buf lay;
      lay.put(3, 1);
      lay.put(1, 1);
      lay.put(d.addr, 8);
      lay.put(d.bytes, 8);
      message(msgs, kLayout, 0, lay);
      meta.pad8();
      const uint64_t oh = here();
      meta.put(1, 1);
      meta.put(0, 1);
      meta.put(4, 2);
      meta.put(1, 4);
      meta.put(msgs.b.size(), 4);
      meta.put(0, 4);
      meta.bytes(msgs.b.data(), msgs.b.size());
      es.push_back({d.name, oh, false, nullptr});
    }
    std::sort(es.begin(), es.end(), [](const Entry &a, const Entry &b) { return a.name < b.name; });
    for (size_t k = 1; k < es.size(); ++k)
      if (es[k].name == es[k - 1].name) return fail(err, "name " + es[k].name + " used twice in one group");
    // local heap data: "" then the names
    Buf heap;
    heap.put(0, 8);
    std::vector<uint64_t> off;
    for (const Entry &e : es) {
      off.push_back(heap.b.size());
      heap.bytes(e.name.c_str(), e.name.size() + 1);
      heap.pad8();
    }
    const size_t nsnod = (es.size() + 2 * kLeafK - 1) / (2 * kLeafK);
    meta.pad8();
    const uint64_t a_heap = here();
    meta.bytes("HEAP", 4);
    meta.put(0, 4);
    meta.put(heap.b.size(), 8);
    meta.put(1, 8);
    meta.put(a_heap + 32, 8);
    meta.bytes(heap.b.data(), heap.b.size());
    std::vector<uint64_t> a_snod;
    for (size_t sn = 0; sn < nsnod; ++sn) {
      meta.pad8();
      a_snod.push_back(here());
      const size_t start = meta.b.size();
      meta.bytes("SNOD", 4);
      meta.put(1, 1);
      meta.put(0, 1);
      const size_t lo = sn * 2 * kLeafK, hi = std::min(es.size(), lo + 2 * kLeafK);
      meta.put(hi - lo, 2);
      for (size_t k = lo; k < hi; ++k) {
        meta.put(off[k], 8);
        meta.put(es[k].oh, 8);
        if (es[k].group) {  // cache type 1: the group's B-tree and heap
          meta.put(1, 4);
          meta.put(0, 4);
          meta.put(es[k].gp->tree, 8);
          meta.put(es[k].gp->heap, 8);
        } else {
          meta.put(0, 4);
          meta.put(0, 4);
          meta.put(0, 16);
        }
      }
      meta.b.resize(start + snod_size, 0);
    }
    meta.pad8();
    const uint64_t a_tree = here();
    {
      const size_t start = meta.b.size();
      meta.bytes("TREE", 4);
      meta.put(0, 1);
      meta.put(0, 1);
      meta.put(nsnod, 2);
      meta.put(kUndef, 8);
      meta.put(kUndef, 8);
      meta.put(0, 8);
      for (size_t sn = 0; sn < nsnod; ++sn) {
        const size_t last = std::min(es.size(), (sn + 1) * 2 * kLeafK) - 1;
        meta.put(a_snod[sn], 8);
        meta.put(off[last], 8);
      }
      meta.b.resize(start + tree_size, 0);
    }
    // the group's object header: its symbol table and its attributes
    Buf msgs;
    Buf st;
    st.put(a_tree, 8);
    st.put(a_heap, 8);
    message(msgs, kSymtab, 0, st);
    for (const Impl::Attr &a : g.attrs) {
      Buf nm, ty = type_of(a.cls, a.size), sp = space_v1({a.n});
      nm.bytes(a.name.c_str(), a.name.size() + 1);
      Buf am;
      am.put(1, 1);
      am.put(0, 1);
      am.put(a.name.size() + 1, 2);
      am.put(ty.b.size(), 2);
      am.put(sp.b.size(), 2);
      nm.pad8();
      ty.pad8();
      sp.pad8();
      am.bytes(nm.b.data(), nm.b.size());
      am.bytes(ty.b.data(), ty.b.size());
      am.bytes(sp.b.data(), sp.b.size());
      am.bytes(a.bytes.data(), a.bytes.size());
      message(msgs, 0x0C, 0, am);
    }
    meta.pad8();
    g.oh = here();
    g.tree = a_tree;
    g.heap = a_heap;
    meta.put(1, 1);
    meta.put(0, 1);
    meta.put(1 + g.attrs.size(), 2);
    meta.put(1, 4);
    meta.put(msgs.b.size(), 4);
    meta.put(0, 4);
    meta.bytes(msgs.b.data(), msgs.b.size());
    return true;
  };
  if (!emit(I.root)) return false;
  // the metadata after the data, then the superblock
  static const uint8_t zeros[8] = {0};
  const uint64_t pad = base - I.eof;
  if ((pad && std::fwrite(zeros, 1, pad, I.f) != pad) ||
      std::fwrite(meta.b.data(), 1, meta.b.size(), I.f) != meta.b.size())
    return fail(err, I.path + ": write failed");
  const uint64_t eof = base + meta.b.size();
  Buf sb;
  sb.bytes(kSig, 8);
  sb.put(0, 4);
  sb.put(0, 1);
  sb.put(8, 1);
  sb.put(8, 1);
  sb.put(0, 1);
  sb.put(kLeafK, 2);
  sb.put(K, 2);
  sb.put(0, 4);
  sb.put(0, 8);
  sb.put(kUndef, 8);
  sb.put(eof, 8);
  sb.put(kUndef, 8);
  sb.put(0, 8);
  sb.put(I.root.oh, 8);
  sb.put(1, 4);
  sb.put(0, 4);
  sb.put(I.root.tree, 8);
  sb.put(I.root.heap, 8);
  const bool ok = std::fseek(I.f, 0, SEEK_SET) == 0 && std::fwrite(sb.b.data(), 1, sb.b.size(), I.f) == sb.b.size();
  const bool closed = std::fclose(I.f) == 0;
  I.f = nullptr;
  if (!ok || !closed) return fail(err, I.path + ": write failed");
  return true;
}

}  // namespace h5
}  // namespace cil

// ---------------------------------------------------------------------------- C ABI
namespace {
thread_local std::string g_h5_err;

cil_status h5_fail(const std::string &m, cil_status s = CIL_ERR_IO) {
  g_h5_err = m;
  return s;
}
}  // namespace

extern "C" {

cil_status cil_h5_shape(const char *path, const char *dataset, int32_t *rank, int64_t dims[8]) {
  if (!path || !dataset || !rank || !dims) return h5_fail("cil_h5_shape: NULL argument", CIL_ERR_CONFIG);
  cil::h5::Reader r;
  cil::h5::Dataset ds;
  std::string err;
  if (!r.open(path, &err) || !r.dataset(dataset, &ds, &err)) return h5_fail(err);
  if (ds.dims.size() > 8) return h5_fail(std::string(dataset) + ": rank above 8");
  *rank = static_cast<int32_t>(ds.dims.size());
  for (size_t k = 0; k < ds.dims.size(); ++k) dims[k] = static_cast<int64_t>(ds.dims[k]);
  return CIL_OK;
}

cil_status cil_h5_read(const char *path, const char *dataset, double *out, int64_t capacity) {
  if (!path || !dataset || (!out && capacity > 0)) return h5_fail("cil_h5_read: NULL argument", CIL_ERR_CONFIG);
  cil::h5::Reader r;
  cil::h5::Dataset ds;
  std::string err;
  std::vector<double> v;
  if (!r.open(path, &err) || !r.dataset(dataset, &ds, &err) || !r.read(ds, &v, &err)) return h5_fail(err);
  if (static_cast<int64_t>(v.size()) > capacity)
    return h5_fail(std::string(dataset) + ": " + std::to_string(v.size()) + " elements, capacity " +
                       std::to_string(capacity),
                   CIL_ERR_CAPACITY);
  std::copy(v.begin(), v.end(), out);
  return CIL_OK;
}

void cil_h5_last_error(char *buf, size_t len) {
  if (!buf || len == 0) return;
  snprintf(buf, len, "%s", g_h5_err.c_str());
}

}  // extern "C"

namespace {

// the datasets of one colony state (outputHDF5Frame), through `put(name, dims, f32 data)` and
// `puti(name, dims, i32 data)`
template <class F32, class I32>
bool put_state(const cil_h5_state *s, F32 put, I32 puti) {
  const uint64_t n = static_cast<uint64_t>(s->ncells), E = static_cast<uint64_t>(s->nelem),
                 D = static_cast<uint64_t>(s->dim);
  const std::vector<double> zv(n * E * D, 0.0), zs(n, 0.0), ze(n * E, 0.0);
  const std::vector<int32_t> zi(n, 0);
  auto pick = [](const double *p, const std::vector<double> &z) { return p ? p : z.data(); };
  const std::vector<uint64_t> vec{n, E, D}, per_elem{n, E}, per_cell{n};
  return put("R", vec, pick(s->pos, zv)) && put("Vel", vec, pick(s->vel, zv)) &&
         put("SigmaCore", per_elem, pick(s->sigma, ze)) && put("F", vec, pick(s->force, zv)) &&
         put("FD", vec, pick(s->force_dis, zv)) && put("FR", vec, pick(s->force_ran, zv)) &&
         put("RHO", per_cell, pick(s->rho, zs)) && put("Theta", per_cell, pick(s->theta, zs)) &&
         put("PR", per_cell, pick(s->pressure, zs)) && puti("State", per_cell, s->state ? s->state : zi.data()) &&
         puti("T0", per_cell, s->t0 ? s->t0 : zi.data()) && put("CpuTime", std::vector<uint64_t>{1}, &s->cpu_time);
}

bool state_ok(const cil_h5_state *s) {
  return s && s->ncells >= 0 && s->nelem >= 1 && (s->dim == 2 || s->dim == 3);
}

}  // namespace

struct cil_h5_frames {
  cil::h5::FrameFile file;
};

extern "C" {

cil_status cil_h5_attr(const char *path, const char *object, const char *name, double *out, int64_t capacity,
                       int64_t *n) {
  if (!path || !object || !name || !n) return h5_fail("cil_h5_attr: NULL argument", CIL_ERR_CONFIG);
  cil::h5::Reader r;
  std::string err;
  std::vector<double> v;
  if (!r.open(path, &err) || !r.attribute(object, name, &v, &err)) return h5_fail(err);
  *n = static_cast<int64_t>(v.size());
  if (*n > capacity) return h5_fail(std::string(name) + ": " + std::to_string(v.size()) + " values", CIL_ERR_CAPACITY);
  std::copy(v.begin(), v.end(), out);
  return CIL_OK;
}

cil_status cil_h5_frames_create(const char *path, int32_t dim, const double *box, double dt, int32_t gts,
                                cil_h5_frames **out) {
  if (!path || !box || !out || (dim != 2 && dim != 3)) return h5_fail("cil_h5_frames_create: bad arguments", CIL_ERR_CONFIG);
  *out = nullptr;
  cil_h5_frames *w = new cil_h5_frames();
  std::string err;
  const bool ok = w->file.create(path, &err) && w->file.attr_f64("params", "dt", {dt}, &err) &&
                  w->file.attr_f64("params", "L", std::vector<double>(box, box + dim), &err) &&
                  w->file.attr_i32("params", "Tdump", {gts}, &err);
  w->file.make_group("snapshots");
  if (!ok) {
    delete w;
    return h5_fail(err);
  }
  *out = w;
  return CIL_OK;
}

cil_status cil_h5_frames_write(cil_h5_frames *w, int32_t frame, int32_t ts, const cil_h5_state *s) {
  if (!w || !state_ok(s) || frame < 0) return h5_fail("cil_h5_frames_write: bad arguments", CIL_ERR_CONFIG);
  const std::string g = "snapshots/t_" + std::to_string(frame);
  std::string err;
  auto put = [&](const char *nm, const std::vector<uint64_t> &dims, const double *d) {
    return w->file.data_f32(g, nm, dims, d, &err);
  };
  auto puti = [&](const char *nm, const std::vector<uint64_t> &dims, const int32_t *d) {
    return w->file.data_i32(g, nm, dims, d, &err);
  };
  if (!w->file.attr_i32(g, "ts", {ts}, &err) || !put_state(s, put, puti)) return h5_fail(err);
  return CIL_OK;
}

cil_status cil_h5_frames_close(cil_h5_frames *w) {
  if (!w) return CIL_OK;
  std::string err;
  const bool ok = w->file.close(&err);
  delete w;
  return ok ? CIL_OK : h5_fail(err);
}

cil_status cil_h5_write_state(const char *path, const cil_h5_state *s) {
  if (!path || !s || s->ncells < 0 || s->nelem < 1 || (s->dim != 2 && s->dim != 3))
    return h5_fail("cil_h5_write_state: bad arguments", CIL_ERR_CONFIG);
  const uint64_t n = static_cast<uint64_t>(s->ncells), E = static_cast<uint64_t>(s->nelem),
                 D = static_cast<uint64_t>(s->dim);
  const std::vector<double> zv(n * E * D, 0.0), zs(n, 0.0), ze(n * E, 0.0);
  const std::vector<int32_t> zi(n, 0);
  auto pick = [](const double *p, const std::vector<double> &z) { return p ? p : z.data(); };
  cil::h5::Writer w;
  std::string err;
  const std::vector<uint64_t> vec{n, E, D}, per_elem{n, E}, per_cell{n};
  bool ok = w.write_f32("R", vec, pick(s->pos, zv), &err) && w.write_f32("Vel", vec, pick(s->vel, zv), &err) &&
            w.write_f32("SigmaCore", per_elem, pick(s->sigma, ze), &err) &&
            w.write_f32("F", vec, pick(s->force, zv), &err) && w.write_f32("FD", vec, pick(s->force_dis, zv), &err) &&
            w.write_f32("FR", vec, pick(s->force_ran, zv), &err) &&
            w.write_f32("RHO", per_cell, pick(s->rho, zs), &err) &&
            w.write_f32("Theta", per_cell, pick(s->theta, zs), &err) &&
            w.write_f32("PR", per_cell, pick(s->pressure, zs), &err) &&
            w.write_i32("State", per_cell, s->state ? s->state : zi.data(), &err) &&
            w.write_i32("T0", per_cell, s->t0 ? s->t0 : zi.data(), &err) &&
            w.write_f32("CpuTime", {1}, &s->cpu_time, &err) && w.save(path, &err);
  return ok ? CIL_OK : h5_fail(err);
}

}  // extern "C"
