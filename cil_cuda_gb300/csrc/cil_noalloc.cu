// cil_bin_elements_noalloc: element binning (the counting sort of cil_bins) for callers
// that cannot allocate device memory.
//
// Who needs it: applications that hand this library only memory they already own — a host
// framework with its own budgeted device pool that forbids outside cudaMalloc, code that
// runs while a CUDA graph is being captured (cudaMalloc is not permitted there), or a
// real-time loop that cannot afford an allocation's latency or failure mid-run. The caller
// passes device input and output buffers; the scratch (keys, bin counts, scan partials)
// lives in file-scope __device__ arrays below, so nothing is allocated by the call.
//
// Limits: at most kMaxElems elements and kMaxBins bins per call (about 8.3 MB of scratch,
// held by every GPU that loads the library until the process exits).
//
// Set-up: the first call on a device looks up the arrays' device addresses with
// cudaGetSymbolAddress (with that device current) and caches them; make that first call
// before any stream capture. Every call shares the same scratch, so calls whose work
// overlaps on the GPU race and must be serialised by the caller (one stream, or events).
// Each call clears the counters it uses before it runs, so the contents left by the
// previous call do not matter.
#include <cuda_runtime.h>

#include <mutex>

#include "cil_internal.cuh"

namespace cil {
namespace {

constexpr int kMaxElems = 1 << 20;
constexpr int kMaxBins = 1 << 20;
constexpr int kNaTile = 256;
constexpr int kNaScan = 1024;  // bins per scan block
constexpr int kMaxDevices = 64;

static __device__ __align__(256) int g_na_key[kMaxElems];
static __device__ __align__(256) int g_na_count[kMaxBins];
static __device__ __align__(256) int g_na_part[kMaxBins / kNaScan];

struct Scratch {
  int *key;
  int *count;
  int *part;
};

struct NaGeom {
  int dim;
  int ns[3];
  double ih[3];
};

__global__ void k_na_clear(int *count, int nbins_pad) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nbins_pad; i += gridDim.x * blockDim.x) count[i] = 0;
}

__global__ void k_na_keys(const double *__restrict__ pos, int n, NaGeom g, int *key, int *count) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  int ls[3] = {0, 0, 0};
  for (int d = 0; d < g.dim; ++d) {
    const double x = pos[static_cast<size_t>(e) * g.dim + d];
    int v = static_cast<int>(__dmul_rn(__dmul_rn(x, g.ih[d]), static_cast<double>(g.ns[d])));
    v = v < g.ns[d] - 1 ? v : g.ns[d] - 1;
    ls[d] = v > 0 ? v : 0;
  }
  const int b = g.dim == 2 ? ls[0] * g.ns[1] + ls[1] : (ls[0] * g.ns[1] + ls[1]) * g.ns[2] + ls[2];
  key[e] = b;
  atomicAdd(count + b, 1);
}

__device__ __forceinline__ int na_block_scan(int v, int *total) {
  __shared__ int ws[kNaTile / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int inc = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) ws[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    int w = lane < kNaTile / 32 ? ws[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += t;
    }
    if (lane < kNaTile / 32) ws[lane] = w;
  }
  __syncthreads();
  const int base = wid > 0 ? ws[wid - 1] : 0;
  *total = ws[kNaTile / 32 - 1];
  __syncthreads();
  return base + inc - v;
}

// per scan block: the sum of its kNaScan counts
__global__ void k_na_partial(const int *count, int *part) {
  const int4 v = reinterpret_cast<const int4 *>(count + blockIdx.x * kNaScan)[threadIdx.x];
  int tot;
  na_block_scan(v.x + v.y + v.z + v.w, &tot);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

// one block: exclusive scan of the partials
__global__ void k_na_scan_parts(int *part, int nparts) {
  int carry = 0;
  for (int base = 0; base < nparts; base += kNaTile) {
    const int i = base + threadIdx.x;
    const int v = i < nparts ? part[i] : 0;
    int tot;
    const int ex = na_block_scan(v, &tot);
    if (i < nparts) part[i] = carry + ex;
    carry += tot;
  }
}

// bin starts; count[] is turned into the per-bin fill cursor (= start)
__global__ void k_na_starts(int *count, const int *part, int nbins, int *bin_start) {
  const int b0 = blockIdx.x * kNaScan + threadIdx.x * 4;
  const int4 v = *reinterpret_cast<const int4 *>(count + b0);
  int tot;
  int s = part[blockIdx.x] + na_block_scan(v.x + v.y + v.z + v.w, &tot);
  const int c[4] = {v.x, v.y, v.z, v.w};
  for (int q = 0; q < 4; ++q) {
    const int b = b0 + q;
    if (b <= nbins) bin_start[b] = s;  // bins past nbins are empty: bin_start[nbins] = n
    count[b] = s;
    s += c[q];
  }
}

__global__ void k_na_scatter(const int *key, int n, int *cursor, int *elems) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const int pos = atomicAdd(cursor + key[e], 1);
  elems[pos] = e;
}

// ascending element ids inside every bin (the order cil_bins reports)
__global__ void k_na_sort(const int *bin_start, int nbins, int *elems) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbins) return;
  const int lo = bin_start[b], hi = bin_start[b + 1];
  for (int i = lo + 1; i < hi; ++i) {
    const int v = elems[i];
    int j = i - 1;
    while (j >= lo && elems[j] > v) {
      elems[j + 1] = elems[j];
      --j;
    }
    elems[j + 1] = v;
  }
}

std::mutex g_na_mutex;
bool g_na_ready[kMaxDevices] = {};
Scratch g_na_scratch[kMaxDevices];

cil_status na_scratch(int dev, Scratch *out) {
  if (dev < 0 || dev >= kMaxDevices) return CIL_ERR_CONFIG;
  std::lock_guard<std::mutex> lock(g_na_mutex);
  if (!g_na_ready[dev]) {
    Scratch s{};
    if (cudaGetSymbolAddress(reinterpret_cast<void **>(&s.key), g_na_key) != cudaSuccess ||
        cudaGetSymbolAddress(reinterpret_cast<void **>(&s.count), g_na_count) != cudaSuccess ||
        cudaGetSymbolAddress(reinterpret_cast<void **>(&s.part), g_na_part) != cudaSuccess)
      return CIL_ERR_CUDA;
    g_na_scratch[dev] = s;
    g_na_ready[dev] = true;
  }
  *out = g_na_scratch[dev];
  return CIL_OK;
}

}  // namespace
}  // namespace cil

extern "C" cil_status cil_bin_elements_noalloc(const double *pos, int32_t n_elems, int32_t dim,
                                               const double *box, double width, int32_t *ns,
                                               int32_t *bin_start, int32_t *elems, int32_t max_bins,
                                               void *stream) {
  using namespace cil;
  if (!pos || !box || !ns || !bin_start || !elems || (dim != 2 && dim != 3) || n_elems < 0 ||
      !(width > 0.0))
    return CIL_ERR_CONFIG;
  if (n_elems > kMaxElems) return CIL_ERR_CAPACITY;
  // grid of LinkListOrtho::get_opt_size + reset (Utils.hpp:872-908)
  NaGeom g{};
  g.dim = dim;
  double mn = box[0];
  for (int d = 1; d < dim; ++d) mn = mn < box[d] ? mn : box[d];
  const double ir = 1.0 / (width + mn * 1.0e-8);
  bool collapse = false;
  long long nb = 1;
  for (int d = 0; d < 3; ++d) {
    g.ns[d] = 1;
    g.ih[d] = 0.0;
  }
  for (int d = 0; d < dim; ++d) {
    if (!(box[d] > 0.0)) return CIL_ERR_CONFIG;
    g.ns[d] = static_cast<int>(box[d] * ir);
    g.ih[d] = 1.0 / box[d];
    collapse = collapse || g.ns[d] < 3;
  }
  if (collapse)
    for (int d = 0; d < dim; ++d) g.ns[d] = 1;
  for (int d = 0; d < dim; ++d) nb *= g.ns[d];
  for (int d = 0; d < 3; ++d) ns[d] = g.ns[d];
  if (nb > kMaxBins || nb > max_bins) return CIL_ERR_CAPACITY;
  const int nbins = static_cast<int>(nb);
  const int nparts = (nbins + 4 + kNaScan - 1) / kNaScan;  // room for the end sentinel
  const int nbins_pad = nparts * kNaScan;
  if (nbins_pad > kMaxBins) return CIL_ERR_CAPACITY;

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CIL_ERR_CUDA;
  Scratch sc{};
  cil_status st = na_scratch(dev, &sc);
  if (st != CIL_OK) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  k_na_clear<<<(nbins_pad + kNaTile - 1) / kNaTile, kNaTile, 0, s>>>(sc.count, nbins_pad);
  if (n_elems > 0) k_na_keys<<<(n_elems + kNaTile - 1) / kNaTile, kNaTile, 0, s>>>(pos, n_elems, g, sc.key, sc.count);
  k_na_partial<<<nparts, kNaTile, 0, s>>>(sc.count, sc.part);
  k_na_scan_parts<<<1, kNaTile, 0, s>>>(sc.part, nparts);
  k_na_starts<<<nparts, kNaTile, 0, s>>>(sc.count, sc.part, nbins, bin_start);
  if (n_elems > 0) k_na_scatter<<<(n_elems + kNaTile - 1) / kNaTile, kNaTile, 0, s>>>(sc.key, n_elems, sc.count, elems);
  k_na_sort<<<(nbins + kNaTile - 1) / kNaTile, kNaTile, 0, s>>>(bin_start, nbins, elems);
  if (cudaGetLastError() != cudaSuccess) return CIL_ERR_CUDA;
  return CIL_OK;
}
