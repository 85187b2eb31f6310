// Frame output in the GSD 1.0 format (HOOMD schema): the file layer cil_gsd_* and the
// device-fed frame writer cil_frame_* (include/cil_gsd.h).
//
// File layer. The on-disk layout is the one the reference's vendored gsd.c writes when
// OutputWriter.cpp opens a file with gsd_create + gsd_open(GSD_OPEN_APPEND):
//   * a 256-byte header at offset 0 (gsd.h:46-59): magic 0x65DF65DF65DF65DF, index location
//     and capacity, name-list location and capacity, schema version, format version 1.0,
//     application[64], schema[64], 80 reserved bytes;
//   * the index right behind it, 128 entries of 32 bytes (frame u64, N u64, location i64,
//     M u32, id u16, type u8, flags u8; gsd.h:65-75), then 128 name-list entries of 64 bytes;
//   * each chunk's data appended at the end of the file when it is written; the frame's index
//     entries written into the index when the frame ends (gsd.c:693-733);
//   * a full index doubles: the old index is copied to the end of the file, zero-filled to the
//     new capacity and the header rewritten with its new place (gsd.c:67-148);
//   * a name gets the next free name-list entry the first time it is used (gsd.c:158-195).
// Readers find the number of index entries as the first entry whose location is 0 and the
// number of frames as the last entry's frame + 1 (gsd.c:355-405), so an unended frame is
// invisible. Files are byte-identical to gsd.c's for the same calls; the tests compare them.
//
// Frame writer. outputGSDFrame (OutputWriter.cpp:505-644) gathers every element from the
// host colony arrays each frame. Here the colony lives in HBM, so one kernel packs the frame
// (positions and velocities as FP32 [E][3], diameters [E]) in the reference element order
// (cell-major, element j of cell i at 2i + j) into a device staging slot; an event hands the
// slot to a second, non-blocking stream that copies it into pinned host memory; a host
// thread waits for that copy and writes the chunks. The caller's next cil_step launches go
// to the handle's stream right after the pack kernel, so the copy and the file writes run
// under the following steps. Two slots: a third frame waits for the oldest to reach the file.
#include <cuda_runtime.h>
#include <errno.h>
#include <fcntl.h>
#include <string.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "cil_gsd.h"
#include "cil_internal.cuh"

// ============================================================================ file layer
namespace {

constexpr uint64_t kGsdMagic = 0x65DF65DF65DF65DFull;
constexpr size_t kHeaderBytes = 256;
constexpr size_t kEntryBytes = 32;
constexpr size_t kNameBytes = 64;
constexpr uint64_t kInitialEntries = 128;
constexpr uint64_t kNameEntries = 128;
constexpr uint16_t kNoId = 0xffff;

size_t type_size(int32_t t) {
  switch (t) {
    case CIL_GSD_UINT8: case CIL_GSD_INT8: return 1;
    case CIL_GSD_UINT16: case CIL_GSD_INT16: return 2;
    case CIL_GSD_UINT32: case CIL_GSD_INT32: case CIL_GSD_FLOAT: return 4;
    case CIL_GSD_UINT64: case CIL_GSD_INT64: case CIL_GSD_DOUBLE: return 8;
    default: return 0;
  }
}

struct IndexEntry {
  uint64_t frame, N;
  int64_t location;
  uint32_t M;
  uint16_t id;
  uint8_t type, flags;
};
static_assert(sizeof(IndexEntry) == kEntryBytes, "GSD index entry is 32 bytes");

// Little-endian serialisation (both hosts that build this library are little-endian).
template <typename T>
void put(unsigned char *p, T v) {
  memcpy(p, &v, sizeof(T));
}

void copy_name(char *dst, const char *src, size_t cap) {  // strncpy(cap - 1) + NUL, zero padded
  memset(dst, 0, cap);
  if (src) strncpy(dst, src, cap - 1);
}

}  // namespace

struct cil_gsd_file {
  int fd = -1;
  // header fields
  uint64_t index_location = kHeaderBytes;
  uint64_t index_entries = kInitialEntries;
  uint64_t namelist_location = kHeaderBytes + kEntryBytes * kInitialEntries;
  uint32_t schema_version = 0;
  char application[64] = {};
  char schema[64] = {};
  // state
  std::vector<std::string> names;   // name list, in id order
  std::vector<IndexEntry> pending;  // entries of the open frame
  uint64_t written = 0;             // index entries on disk
  uint64_t frame = 0;               // frames ended
  int64_t file_size = 0;
  std::string err;

  cil_status io_fail(const char *what) {
    err = std::string(what) + ": " + strerror(errno);
    return CIL_ERR_IO;
  }

  bool pwrite_all(const void *data, size_t n, int64_t at) {
    const unsigned char *p = static_cast<const unsigned char *>(data);
    while (n > 0) {
      const ssize_t w = ::pwrite(fd, p, n, static_cast<off_t>(at));
      if (w < 0 && errno == EINTR) continue;
      if (w <= 0) return false;
      p += w;
      n -= static_cast<size_t>(w);
      at += w;
    }
    return true;
  }

  bool pread_all(void *data, size_t n, int64_t at) {
    unsigned char *p = static_cast<unsigned char *>(data);
    while (n > 0) {
      const ssize_t r = ::pread(fd, p, n, static_cast<off_t>(at));
      if (r < 0 && errno == EINTR) continue;
      if (r <= 0) return false;
      p += r;
      n -= static_cast<size_t>(r);
      at += r;
    }
    return true;
  }

  bool write_header() {
    unsigned char b[kHeaderBytes];
    memset(b, 0, sizeof(b));
    put<uint64_t>(b + 0, kGsdMagic);
    put<uint64_t>(b + 8, index_location);
    put<uint64_t>(b + 16, index_entries);
    put<uint64_t>(b + 24, namelist_location);
    put<uint64_t>(b + 32, kNameEntries);
    put<uint32_t>(b + 40, schema_version);
    put<uint32_t>(b + 44, CIL_GSD_VERSION(1, 0));
    memcpy(b + 48, application, 64);
    memcpy(b + 112, schema, 64);
    return pwrite_all(b, sizeof(b), 0);
  }

  // Name -> id; new names take the next name-list entry while there is one (gsd.c:158-195).
  // The lookup compares the caller's name, untruncated, as gsd.c does: a name of 64 or more
  // characters never matches its stored, truncated form and takes a new entry on every call.
  uint16_t name_id(const char *name, cil_status *st) {
    for (size_t i = 0; i < names.size(); ++i)
      if (strncmp(name, names[i].c_str(), kNameBytes) == 0) return static_cast<uint16_t>(i);
    char key[kNameBytes];
    copy_name(key, name, kNameBytes);
    if (names.size() >= kNameEntries) return kNoId;
    const int64_t at = static_cast<int64_t>(namelist_location + kNameBytes * names.size());
    if (!pwrite_all(key, kNameBytes, at)) {
      *st = io_fail("gsd name list write");
      return kNoId;
    }
    names.emplace_back(key);
    return static_cast<uint16_t>(names.size() - 1);
  }

  // Doubles the index at the end of the file (gsd.c:67-148, append-mode branch).
  cil_status grow_index() {
    const uint64_t old_bytes = index_entries * kEntryBytes;
    const uint64_t new_bytes = 2 * old_bytes;
    const int64_t new_loc = file_size;
    std::vector<unsigned char> buf(16384);
    uint64_t done = 0;
    while (done < old_bytes) {
      const size_t n = static_cast<size_t>(std::min<uint64_t>(buf.size(), old_bytes - done));
      if (!pread_all(buf.data(), n, static_cast<int64_t>(index_location + done))) return io_fail("gsd index read");
      if (!pwrite_all(buf.data(), n, new_loc + static_cast<int64_t>(done))) return io_fail("gsd index write");
      done += n;
    }
    std::fill(buf.begin(), buf.end(), 0);
    while (done < new_bytes) {
      const size_t n = static_cast<size_t>(std::min<uint64_t>(buf.size(), new_bytes - done));
      if (!pwrite_all(buf.data(), n, new_loc + static_cast<int64_t>(done))) return io_fail("gsd index write");
      done += n;
    }
    index_location = static_cast<uint64_t>(new_loc);
    index_entries *= 2;
    file_size = new_loc + static_cast<int64_t>(new_bytes);
    if (!write_header()) return io_fail("gsd header write");
    return CIL_OK;
  }
};

extern "C" {

cil_status cil_gsd_create(const char *path, const char *application, const char *schema, uint32_t schema_version,
                          cil_gsd_file **out) {
  if (!path || !out) return CIL_ERR_CONFIG;
  *out = nullptr;
  cil_gsd_file *f = new cil_gsd_file();
  f->fd = ::open(path, O_RDWR | O_CREAT | O_TRUNC, S_IRUSR | S_IWUSR | S_IRGRP | S_IWGRP);
  if (f->fd < 0) {
    delete f;
    return CIL_ERR_IO;
  }
  copy_name(f->application, application ? application : "", 64);
  copy_name(f->schema, schema ? schema : "", 64);
  f->schema_version = schema_version;
  std::vector<unsigned char> zeros(kEntryBytes * kInitialEntries + kNameBytes * kNameEntries, 0);
  if (!f->write_header() || !f->pwrite_all(zeros.data(), zeros.size(), kHeaderBytes)) {
    ::close(f->fd);
    delete f;
    return CIL_ERR_IO;
  }
  f->file_size = static_cast<int64_t>(kHeaderBytes + zeros.size());
  *out = f;
  return CIL_OK;
}

cil_status cil_gsd_write_chunk(cil_gsd_file *f, const char *name, int32_t type, uint64_t N, uint32_t M,
                               const void *data) {
  if (!f) return CIL_ERR_CONFIG;
  const size_t es = type_size(type);
  if (!data || !name || N == 0 || M == 0 || es == 0) {
    f->err = "cil_gsd_write_chunk: empty chunk, NULL data or unknown type";
    return CIL_ERR_CONFIG;
  }
  cil_status st = CIL_OK;
  IndexEntry e{};
  e.frame = f->frame;
  e.id = f->name_id(name, &st);
  if (st != CIL_OK) return st;
  e.type = static_cast<uint8_t>(type);
  e.N = N;
  e.M = M;
  e.location = f->file_size;
  const size_t bytes = static_cast<size_t>(N) * M * es;
  if (!f->pwrite_all(data, bytes, e.location)) return f->io_fail("gsd chunk write");
  f->file_size += static_cast<int64_t>(bytes);
  if (f->written + f->pending.size() >= f->index_entries) {
    st = f->grow_index();
    if (st != CIL_OK) return st;
  }
  f->pending.push_back(e);
  return CIL_OK;
}

cil_status cil_gsd_end_frame(cil_gsd_file *f) {
  if (!f) return CIL_ERR_CONFIG;
  f->frame += 1;
  if (!f->pending.empty()) {
    const int64_t at = static_cast<int64_t>(f->index_location + kEntryBytes * f->written);
    if (!f->pwrite_all(f->pending.data(), kEntryBytes * f->pending.size(), at)) return f->io_fail("gsd index write");
    f->written += f->pending.size();
    f->pending.clear();
  }
  return CIL_OK;
}

uint64_t cil_gsd_nframes(const cil_gsd_file *f) { return f ? f->frame : 0; }

cil_status cil_gsd_close(cil_gsd_file *f) {
  if (!f) return CIL_OK;
  const int r = ::close(f->fd);
  delete f;
  return r == 0 ? CIL_OK : CIL_ERR_IO;
}

void cil_gsd_last_error(const cil_gsd_file *f, char *buf, size_t len) {
  if (!buf || len == 0) return;
  const char *m = f ? f->err.c_str() : "";
  snprintf(buf, len, "%s", m);
}

}  // extern "C"

// ============================================================================ pack kernel
namespace cil {
namespace {

template <int D>
__global__ void __launch_bounds__(kTile) k_frame_pack(int E, size_t SS, int elem_base, const int *__restrict__ slot_of,
                                                     const double *__restrict__ x, const double *__restrict__ vel,
                                                     const double *__restrict__ sigma_c, double h0, double h1,
                                                     double h2, float z0, float z1, float *__restrict__ out) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  const int s = slot_of[elem_base + e];
  const double x0 = x[s], x1 = x[SS + s];
  const double v0 = vel[s], v1 = vel[SS + s];
  const double dia = sigma_c[elem_base + e];
  float *pos = out + 3 * static_cast<size_t>(e);
  float *v = out + 3 * static_cast<size_t>(E) + 3 * static_cast<size_t>(e);
  // gsdBufferVectorShiftScale2D/3D (OutputWriter.cpp:126-153): the shift in FP64, then one
  // rounding to FP32, as the host assignment to float does.
  pos[0] = static_cast<float>(x0 - h0);
  pos[1] = static_cast<float>(x1 - h1);
  v[0] = static_cast<float>(v0);
  v[1] = static_cast<float>(v1);
  if (D == 3) {
    pos[2] = static_cast<float>(x[2 * SS + s] - h2);
    v[2] = static_cast<float>(vel[2 * SS + s]);
  } else {
    pos[2] = (e & 1) ? z1 : z0;  // zhack[j] (OutputWriter.cpp:607-610)
    v[2] = 0.0f;                  // gsdBufferVector2D (OutputWriter.cpp:156-166)
  }
  out[6 * static_cast<size_t>(E) + e] = static_cast<float>(dia);
}

}  // namespace

void launch_frame_pack(const FrameSource &s, const double half[3], const float zj[2], float *out, cudaStream_t st) {
  const int E = 2 * s.ncells;
  if (E <= 0) return;
  const int grid = (E + kTile - 1) / kTile;
  const int base = 2 * s.cell_base;
  if (s.dim == 3)
    k_frame_pack<3><<<grid, kTile, 0, st>>>(E, s.SS, base, s.slot_of, s.x, s.vel, s.sigma_c, half[0], half[1],
                                            half[2], zj[0], zj[1], out);
  else
    k_frame_pack<2><<<grid, kTile, 0, st>>>(E, s.SS, base, s.slot_of, s.x, s.vel, s.sigma_c, half[0], half[1],
                                            half[2], zj[0], zj[1], out);
}

}  // namespace cil

// ============================================================================ frame writer
namespace {

using Clock = std::chrono::steady_clock;

double ms_since(Clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
}

constexpr int kSlots = 2;
constexpr int kTypeChars = 63;  // particles/types row width (OutputWriter.cpp:540)

struct FrameJob {
  int slot;
  int E;
  uint64_t step;
  bool types, per_elem, charge;
};

}  // namespace

struct cil_frame_writer {
  cil_handle *h = nullptr;
  int colony = 0;
  int device = 0;
  cil_gsd_file *file = nullptr;
  int dim = 2;
  int divide = 0, dying = 0;
  float box[6] = {0, 0, 0, 0, 0, 0};
  double lz_opt = 0.0;
  bool box_ready = false;
  double half[3] = {0, 0, 0};
  float zj[2] = {0, 0};
  int flags = 0;
  std::vector<char> types;  // [2][63]
  cudaStream_t copy = nullptr;
  cudaEvent_t begin[kSlots] = {nullptr, nullptr};  // before the pack kernel
  cudaEvent_t packed[kSlots] = {nullptr, nullptr};
  cudaEvent_t copied[kSlots] = {nullptr, nullptr};
  float *d_buf[kSlots] = {nullptr, nullptr};
  float *h_buf[kSlots] = {nullptr, nullptr};
  size_t cap[kSlots] = {0, 0};  // floats per slot
  bool busy[kSlots] = {false, false};
  int next_slot = 0;
  // writer thread
  std::thread th;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<FrameJob> q;
  bool stop = false;
  cil_status err_st = CIL_OK;
  std::string err;
  // thread-owned scratch
  std::vector<uint32_t> typeid_buf;
  std::vector<float> charge_buf, mass_buf;  // the constant chunks, filled when the count grows
  // counters
  int64_t queued = 0, done = 0, d2h_bytes = 0, file_bytes = 0;
  double enqueue_ms = 0, slot_wait_ms = 0, write_ms = 0, pack_ms = 0, copy_ms = 0;

  void set_error(cil_status s, const std::string &m) {  // caller holds mu
    if (err_st == CIL_OK) {
      err_st = s;
      err = m;
    }
  }

  cil_status write_job(const FrameJob &j) {
    cil_gsd_file *f = file;
    const float *pos = h_buf[j.slot];
    const float *vel = pos + 3 * static_cast<size_t>(j.E);
    const float *dia = pos + 6 * static_cast<size_t>(j.E);
    const uint64_t step = j.step;
    const uint8_t dims = 3;  // MAX_DIM (OutputWriter.cpp:508)
    const uint32_t n = static_cast<uint32_t>(j.E);
    cil_status st;
#define CIL_W(call)            \
  do {                         \
    st = (call);               \
    if (st != CIL_OK) return st; \
  } while (0)
    CIL_W(cil_gsd_write_chunk(f, "configuration/step", CIL_GSD_UINT64, 1, 1, &step));
    CIL_W(cil_gsd_write_chunk(f, "configuration/dimensions", CIL_GSD_UINT8, 1, 1, &dims));
    CIL_W(cil_gsd_write_chunk(f, "configuration/box", CIL_GSD_FLOAT, 6, 1, box));
    CIL_W(cil_gsd_write_chunk(f, "particles/N", CIL_GSD_UINT32, 1, 1, &n));
    if (j.types) CIL_W(cil_gsd_write_chunk(f, "particles/types", CIL_GSD_INT8, 2, kTypeChars, types.data()));
    if (j.E > 0) {
      const size_t E = static_cast<size_t>(j.E);
      if (j.per_elem) {
        CIL_W(cil_gsd_write_chunk(f, "particles/Z", CIL_GSD_FLOAT, E, 1, dia));
        CIL_W(cil_gsd_write_chunk(f, "particles/diameter", CIL_GSD_FLOAT, E, 1, dia));
        if (typeid_buf.size() < E) {
          typeid_buf.resize(E);
          for (size_t e = 0; e < E; ++e) typeid_buf[e] = static_cast<uint32_t>(e & 1);  // elemType[j]
        }
        CIL_W(cil_gsd_write_chunk(f, "particles/typeid", CIL_GSD_UINT32, E, 1, typeid_buf.data()));
      }
      if (j.charge) {
        if (charge_buf.size() < E) charge_buf.assign(E, -1.0f);  // cellTRho, never set by the two-element model
        CIL_W(cil_gsd_write_chunk(f, "particles/charge", CIL_GSD_FLOAT, E, 1, charge_buf.data()));
      }
      CIL_W(cil_gsd_write_chunk(f, "particles/position", CIL_GSD_FLOAT, E, 3, pos));
      CIL_W(cil_gsd_write_chunk(f, "particles/velocity", CIL_GSD_FLOAT, E, 3, vel));
      if (mass_buf.size() < E) mass_buf.assign(E, 0.0f);  // pressure
      CIL_W(cil_gsd_write_chunk(f, "particles/mass", CIL_GSD_FLOAT, E, 1, mass_buf.data()));
    }
#undef CIL_W
    return cil_gsd_end_frame(f);
  }

  void run() {
    cudaSetDevice(device);
    for (;;) {
      FrameJob j;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [&] { return stop || !q.empty(); });
        if (q.empty()) return;
        j = q.front();
        q.pop_front();
      }
      const auto t0 = Clock::now();
      cil_status st = CIL_OK;
      std::string m;
      const cudaError_t ce = cudaEventSynchronize(copied[j.slot]);
      float pk = 0.0f, cp = 0.0f;
      if (ce == cudaSuccess) {
        cudaEventElapsedTime(&pk, begin[j.slot], packed[j.slot]);
        cudaEventElapsedTime(&cp, packed[j.slot], copied[j.slot]);
      }
      if (ce != cudaSuccess) {
        st = CIL_ERR_CUDA;
        m = std::string("frame copy: ") + cudaGetErrorString(ce);
      } else {
        bool skip;
        {
          std::lock_guard<std::mutex> lk(mu);
          skip = err_st != CIL_OK;  // after a failure the file is left as it was
        }
        if (!skip) {
          st = write_job(j);
          if (st != CIL_OK) m = file->err;
        }
      }
      const double ms = ms_since(t0);
      {
        std::lock_guard<std::mutex> lk(mu);
        if (st != CIL_OK) set_error(st, m);
        busy[j.slot] = false;
        done += 1;
        file_bytes = file->file_size;
        write_ms += ms;
        pack_ms += pk;
        copy_ms += cp;
      }
      cv.notify_all();
    }
  }

  cil_status status() {
    std::lock_guard<std::mutex> lk(mu);
    return err_st;
  }

  cil_status flush() {
    std::unique_lock<std::mutex> lk(mu);
    cv.wait(lk, [&] { return q.empty() && !busy[0] && !busy[1]; });
    return err_st;
  }

  void release() {
    if (th.joinable()) {
      {
        std::lock_guard<std::mutex> lk(mu);
        stop = true;
      }
      cv.notify_all();
      th.join();
    }
    if (copy) cudaStreamSynchronize(copy);
    for (int s = 0; s < kSlots; ++s) {
      if (begin[s]) cudaEventDestroy(begin[s]);
      if (packed[s]) cudaEventDestroy(packed[s]);
      if (copied[s]) cudaEventDestroy(copied[s]);
      if (d_buf[s]) cudaFree(d_buf[s]);
      if (h_buf[s]) cudaFreeHost(h_buf[s]);
    }
    if (copy) cudaStreamDestroy(copy);
  }
};

namespace {

cil_status writer_fail(cil_frame_writer *w, cil_status s, const std::string &m) {
  std::lock_guard<std::mutex> lk(w->mu);
  w->set_error(s, m);
  return s;
}

}  // namespace

extern "C" {

cil_status cil_frame_open(cil_handle *h, int32_t colony, const char *path, const cil_frame_options *opt,
                          cil_frame_writer **out) {
  if (!h || !path || !out) return CIL_ERR_CONFIG;
  *out = nullptr;
  cil::FrameSource s{};
  cil_status st = cil::frame_layout(h, colony, &s);
  if (st != CIL_OK) return st;
  if (cudaSetDevice(s.device) != cudaSuccess) {
    cudaGetLastError();
    return CIL_ERR_CUDA;
  }
  cil_frame_options o{};
  if (opt) o = *opt;
  cil_frame_writer *w = new cil_frame_writer();
  w->h = h;
  w->colony = colony;
  w->device = s.device;
  w->dim = s.dim;
  w->divide = s.divide;
  w->dying = s.dying;
  w->flags = o.flags;
  // 2D box z: the option, else the largest uploaded diameter, read at the first frame
  w->lz_opt = o.lz;
  w->box[0] = static_cast<float>(s.box[0]);
  w->box[1] = static_cast<float>(s.box[1]);
  w->box[2] = static_cast<float>(s.dim == 3 ? s.box[2] : o.lz);
  for (int d = 0; d < 3; ++d) w->half[d] = 0.5 * s.box[d];
  // zhack[j] = j * (-0.01 * units.Length) in FP64, then FP32 (OutputWriter.cpp:607-610);
  // element 0 lands on -0.0.
  const double unit = o.length_unit > 0.0 ? o.length_unit : 1.0;
  for (int j = 0; j < 2; ++j) w->zj[j] = static_cast<float>(static_cast<double>(j) * (-0.01 * unit));
  // "<cell>_<element tag>", at most 62 characters, zero padded (OutputWriter.cpp:538-556)
  const char *cell = o.cell_name ? o.cell_name : "A";
  const char *tags[2] = {o.elem_names[0] ? o.elem_names[0] : "BACK", o.elem_names[1] ? o.elem_names[1] : "FRONT"};
  w->types.assign(2 * kTypeChars, 0);
  for (int j = 0; j < 2; ++j) snprintf(w->types.data() + j * kTypeChars, kTypeChars, "%s_%s", cell, tags[j]);

  st = cil_gsd_create(path, "CIL", "hoomd", CIL_GSD_VERSION(1, 1), &w->file);
  if (st != CIL_OK) {
    delete w;
    return st;
  }
  bool ok = cudaStreamCreateWithFlags(&w->copy, cudaStreamNonBlocking) == cudaSuccess;
  for (int k = 0; ok && k < kSlots; ++k)
    ok = cudaEventCreate(&w->begin[k]) == cudaSuccess && cudaEventCreate(&w->packed[k]) == cudaSuccess &&
         cudaEventCreate(&w->copied[k]) == cudaSuccess;
  // staging for the colony's capacity, allocated here so that frames never allocate
  const size_t cap = 7 * static_cast<size_t>(2 * s.capacity) + 1024;
  for (int k = 0; ok && k < kSlots; ++k) {
    ok = cudaMalloc(&w->d_buf[k], cap * sizeof(float)) == cudaSuccess &&
         cudaHostAlloc(&w->h_buf[k], cap * sizeof(float), cudaHostAllocDefault) == cudaSuccess;
    if (ok) w->cap[k] = cap;
  }
  if (!ok) {
    cudaGetLastError();
    w->release();
    cil_gsd_close(w->file);
    delete w;
    return CIL_ERR_CUDA;
  }
  w->th = std::thread([w] { w->run(); });
  *out = w;
  return CIL_OK;
}

cil_status cil_frame_write(cil_frame_writer *w, int64_t step, int64_t *frame) {
  if (!w) return CIL_ERR_CONFIG;
  const auto t0 = Clock::now();
  cil_status st = w->status();
  if (st != CIL_OK) return st;
  cil::FrameSource s{};
  st = cil::frame_source(w->h, w->colony, &s);
  if (st != CIL_OK) return st;  // the handle holds the message
  if (!w->box_ready) {  // before any frame is queued, so the writer thread never sees it change
    if (w->dim == 2 && !(w->lz_opt > 0.0)) w->box[2] = static_cast<float>(s.sigma_max);  // lz2d
    w->box_ready = true;
  }
  const int slot = w->next_slot;
  {
    const auto tw = Clock::now();
    std::unique_lock<std::mutex> lk(w->mu);
    w->cv.wait(lk, [&] { return !w->busy[slot] || w->err_st != CIL_OK; });
    w->slot_wait_ms += ms_since(tw);
    if (w->err_st != CIL_OK) return w->err_st;
  }
  const int E = 2 * s.ncells;
  const size_t need = 7 * static_cast<size_t>(E);
  if (need > w->cap[slot]) {  // the slot is idle: its last copy has been waited for
    const size_t cap = need + need / 4 + 1024;
    if (w->d_buf[slot]) cudaFree(w->d_buf[slot]);
    if (w->h_buf[slot]) cudaFreeHost(w->h_buf[slot]);
    w->d_buf[slot] = nullptr;
    w->h_buf[slot] = nullptr;
    w->cap[slot] = 0;
    if (cudaMalloc(&w->d_buf[slot], cap * sizeof(float)) != cudaSuccess ||
        cudaHostAlloc(&w->h_buf[slot], cap * sizeof(float), cudaHostAllocDefault) != cudaSuccess) {
      cudaGetLastError();
      return writer_fail(w, CIL_ERR_CUDA, "out of memory (frame staging)");
    }
    w->cap[slot] = cap;
  }
  cudaError_t ce = cudaEventRecord(w->begin[slot], s.stream);
  if (ce == cudaSuccess && E > 0) {
    cil::launch_frame_pack(s, w->half, w->zj, w->d_buf[slot], s.stream);
    ce = cudaGetLastError();
  }
  if (ce == cudaSuccess) ce = cudaEventRecord(w->packed[slot], s.stream);
  if (ce == cudaSuccess) ce = cudaStreamWaitEvent(w->copy, w->packed[slot], 0);
  if (ce == cudaSuccess && E > 0)
    ce = cudaMemcpyAsync(w->h_buf[slot], w->d_buf[slot], need * sizeof(float), cudaMemcpyDeviceToHost, w->copy);
  if (ce == cudaSuccess) ce = cudaEventRecord(w->copied[slot], w->copy);
  if (ce != cudaSuccess) return writer_fail(w, CIL_ERR_CUDA, std::string("frame enqueue: ") + cudaGetErrorString(ce));
  const uint64_t st_step = static_cast<uint64_t>(step < 0 ? s.ts : step);
  FrameJob j{};
  j.slot = slot;
  j.E = E;
  j.step = st_step;
  j.types = st_step == 0 || ((w->flags & CIL_FRAME_TYPES_IN_FIRST) && w->queued == 0);
  j.per_elem = w->divide || w->dying || st_step == 0;
  j.charge = w->divide != 0;
  int64_t idx;
  {
    std::lock_guard<std::mutex> lk(w->mu);
    w->busy[slot] = true;
    w->q.push_back(j);
    idx = w->queued++;
    w->d2h_bytes += static_cast<int64_t>(need * sizeof(float));
    w->enqueue_ms += ms_since(t0);
  }
  w->cv.notify_all();
  w->next_slot = (slot + 1) % kSlots;
  if (frame) *frame = idx;
  return CIL_OK;
}

cil_status cil_frame_flush(cil_frame_writer *w) {
  if (!w) return CIL_ERR_CONFIG;
  return w->flush();
}

cil_status cil_frame_close(cil_frame_writer *w) {
  if (!w) return CIL_OK;
  cil_status st = w->flush();
  w->release();
  const cil_status cs = cil_gsd_close(w->file);
  delete w;
  return st != CIL_OK ? st : cs;
}

cil_status cil_frame_get_stats(const cil_frame_writer *w, cil_frame_stats *out) {
  if (!w || !out) return CIL_ERR_CONFIG;
  cil_frame_writer *m = const_cast<cil_frame_writer *>(w);
  std::lock_guard<std::mutex> lk(m->mu);
  out->frames_queued = w->queued;
  out->frames_written = w->done;
  out->d2h_bytes = w->d2h_bytes;
  out->file_bytes = w->file_bytes;
  out->enqueue_ms = w->enqueue_ms;
  out->slot_wait_ms = w->slot_wait_ms;
  out->write_ms = w->write_ms;
  out->pack_ms = w->pack_ms;
  out->copy_ms = w->copy_ms;
  return CIL_OK;
}

void cil_frame_last_error(const cil_frame_writer *w, char *buf, size_t len) {
  if (!buf || len == 0) return;
  if (!w) {
    buf[0] = 0;
    return;
  }
  cil_frame_writer *m = const_cast<cil_frame_writer *>(w);
  std::lock_guard<std::mutex> lk(m->mu);
  snprintf(buf, len, "%s", w->err.c_str());
}

}  // extern "C"
