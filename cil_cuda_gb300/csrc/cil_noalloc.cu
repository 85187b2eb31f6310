// cil_bin_elements_noalloc: element binning (the counting sort of cil_bins) for callers
// that cannot allocate device memory.
//
// Who needs it: applications that hand this library only memory they already own — a host
// framework with its own budgeted device pool that forbids outside cudaMalloc, or a real-time
// loop that cannot afford an allocation's latency or its failure mid-run. The caller passes
// device input and output buffers; the scratch (bin keys, the radix pass's packed ids, bin
// counts, per-tile digit histograms, scan partials) lives in file-scope __device__ arrays
// below, so nothing is allocated by the call.
//
// Order inside a bin: ascending element id, as cil_bins reports it. It comes out of a stable
// LSD radix sort of the bin keys (keys are produced in element order): one pass of 10-bit
// digits when the grid has at most 1024 bins, two passes otherwise. Each pass is a per-tile
// digit histogram, one exclusive scan over (digit, tile), and a scatter in which each tile
// ranks its elements stably with warp matches. The work is linear in the element count
// whatever the bin occupancy; a grid collapsed to one bin costs the same as any other.
//
// Limits: at most kMaxElems elements and kMaxBins bins per call (about 14.7 MB of scratch,
// held by every GPU that loads the library until the process exits).
//
// Set-up: the first call on a device looks up the arrays' device addresses with
// cudaGetSymbolAddress (with that device current) and caches them; make that first call
// before any stream capture. Every call shares the same scratch, so calls whose work
// overlaps on the GPU race and must be serialised by the caller (one stream, or events).
// Each call clears or overwrites every scratch word it reads before it runs, so the contents
// left by the previous call do not matter.
#include <cuda_runtime.h>

#include <mutex>

#include "cil_internal.cuh"

namespace cil {
namespace {

constexpr int kMaxElems = 1 << 20;
constexpr int kMaxBins = 1 << 20;
constexpr int kNaTile = 256;
constexpr int kNaScan = 1024;        // entries per scan block
constexpr int kDigitBits = 10;       // radix digit: 1024 buckets
constexpr int kDigits = 1 << kDigitBits;
constexpr int kRadixTile = 2048;     // elements per radix tile (one warp, 64 chunks of 32)
constexpr int kMaxTiles = kMaxElems / kRadixTile;
constexpr int kIdBits = 20;          // element id field of a packed pass-0 entry (kMaxElems = 2^20)
constexpr int kMaxDevices = 64;
static_assert(kMaxElems <= (1 << kIdBits), "element ids must fit the packed field");
static_assert(kMaxBins <= kDigits * kDigits, "two radix passes must cover every bin key");

static __device__ __align__(256) int g_na_key[kMaxElems];                 // bin key per element
static __device__ __align__(256) int g_na_alt[kMaxElems];                 // pass 0 out: id | high digit << 20
static __device__ __align__(256) int g_na_count[kMaxBins + kNaScan];      // bin counts (+ end sentinel room)
static __device__ __align__(256) int g_na_hist[kDigits * kMaxTiles];      // [digit][tile] counts -> offsets
static __device__ __align__(256) int g_na_part[kMaxBins / kNaScan + 1];   // scan partials

struct Scratch {
  int *key;
  int *alt;
  int *count;
  int *hist;
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

// bin starts from the bin counts and their scanned scan-block sums
__global__ void k_na_starts(const int *count, const int *part, int nbins, int *bin_start) {
  const int b0 = blockIdx.x * kNaScan + threadIdx.x * 4;
  const int4 v = *reinterpret_cast<const int4 *>(count + b0);
  int tot;
  int s = part[blockIdx.x] + na_block_scan(v.x + v.y + v.z + v.w, &tot);
  const int c[4] = {v.x, v.y, v.z, v.w};
  for (int q = 0; q < 4; ++q) {
    const int b = b0 + q;
    if (b <= nbins) bin_start[b] = s;  // bins past nbins are empty: bin_start[nbins] = n
    s += c[q];
  }
}

// in-place exclusive scan of a count array whose scan-block sums are already scanned in part[]
__global__ void k_na_offsets(int *v, const int *part) {
  int4 *p = reinterpret_cast<int4 *>(v + blockIdx.x * kNaScan) + threadIdx.x;
  const int4 c = *p;
  int tot;
  const int s = part[blockIdx.x] + na_block_scan(c.x + c.y + c.z + c.w, &tot);
  *p = make_int4(s, s + c.x, s + c.x + c.y, s + c.x + c.y + c.z);
}

// radix digit of element i in pass `pass` (0: low 10 bits of the key, 1: high 10 bits, read
// from the packed pass-0 output)
__device__ __forceinline__ int na_digit(int pass, const int *src, int i) {
  const int v = src[i];
  return pass == 0 ? (v & (kDigits - 1)) : (v >> kIdBits);
}

// per radix tile: digit histogram, written digit-major (hist[digit * ntiles + tile]) so that
// one exclusive scan gives every (digit, tile) its first output position
__global__ void __launch_bounds__(32) k_na_hist(int pass, const int *src, int n, int ntiles, int *hist) {
  __shared__ int h[kDigits];
  const int lane = threadIdx.x;
  for (int d = lane; d < kDigits; d += 32) h[d] = 0;
  __syncwarp();
  const int i0 = blockIdx.x * kRadixTile;
  const int i1 = min(n, i0 + kRadixTile);
  for (int i = i0 + lane; i < i1; i += 32) atomicAdd(h + na_digit(pass, src, i), 1);
  __syncwarp();
  for (int d = lane; d < kDigits; d += 32) hist[d * ntiles + blockIdx.x] = h[d];
}

// per radix tile, in element order 32 at a time: each element's place is its (digit, tile)
// offset plus the elements of the same digit before it in the tile (warp match + popcount),
// so the scatter is stable. Pass 0 of two writes id | high digit << 20 into alt; the last pass
// writes element ids into the caller's array.
__global__ void __launch_bounds__(32) k_na_rank_scatter(int pass, int last, const int *src, int n, int ntiles,
                                                        const int *hist, int *alt, int *elems) {
  __shared__ int cur[kDigits];
  const int lane = threadIdx.x;
  for (int d = lane; d < kDigits; d += 32) cur[d] = hist[d * ntiles + blockIdx.x];
  __syncwarp();
  const unsigned lt = (1u << lane) - 1u;
  const int i0 = blockIdx.x * kRadixTile;
  const int i1 = min(n, i0 + kRadixTile);
  for (int base = i0; base < i1; base += 32) {
    const int i = base + lane;
    const bool valid = i < i1;
    const int v = valid ? src[i] : 0;
    const int d = valid ? (pass == 0 ? (v & (kDigits - 1)) : (v >> kIdBits)) : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int at = valid ? cur[d] : 0;  // every lane reads before any leader advances
    __syncwarp();
    if (valid && lane == __ffs(peers) - 1) cur[d] = at + __popc(peers);
    __syncwarp();
    if (valid) {
      const int pos = at + __popc(peers & lt);
      const int id = pass == 0 ? i : (v & ((1 << kIdBits) - 1));
      if (last)
        elems[pos] = id;
      else
        alt[pos] = id | ((v >> kDigitBits) << kIdBits);
    }
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
        cudaGetSymbolAddress(reinterpret_cast<void **>(&s.alt), g_na_alt) != cudaSuccess ||
        cudaGetSymbolAddress(reinterpret_cast<void **>(&s.count), g_na_count) != cudaSuccess ||
        cudaGetSymbolAddress(reinterpret_cast<void **>(&s.hist), g_na_hist) != cudaSuccess ||
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
    // more than kMaxBins bins along one axis never fit (and would overflow the int cast)
    if (!(box[d] * ir < static_cast<double>(kMaxBins) + 1.0)) return CIL_ERR_CAPACITY;
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
  const int nparts = (nbins + 1 + kNaScan - 1) / kNaScan;  // room for the end sentinel
  const int nbins_pad = nparts * kNaScan;                   // <= kMaxBins + kNaScan

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
  if (n_elems > 0) {
    // stable radix sort of the keys by bin: one pass of 10-bit digits for grids of at most
    // 1024 bins, two otherwise (ntiles <= 512, so the histogram scan has <= 512 blocks)
    const int ntiles = (n_elems + kRadixTile - 1) / kRadixTile;
    const int npass = nbins <= kDigits ? 1 : 2;
    const int hparts = ntiles;  // kDigits * ntiles entries, kNaScan per scan block
    for (int pass = 0; pass < npass; ++pass) {
      const int *src = pass == 0 ? sc.key : sc.alt;
      k_na_hist<<<ntiles, 32, 0, s>>>(pass, src, n_elems, ntiles, sc.hist);
      k_na_partial<<<hparts, kNaTile, 0, s>>>(sc.hist, sc.part);
      k_na_scan_parts<<<1, kNaTile, 0, s>>>(sc.part, hparts);
      k_na_offsets<<<hparts, kNaTile, 0, s>>>(sc.hist, sc.part);
      k_na_rank_scatter<<<ntiles, 32, 0, s>>>(pass, pass == npass - 1, src, n_elems, ntiles, sc.hist, sc.alt,
                                              elems);
    }
  }
  if (cudaGetLastError() != cudaSuccess) return CIL_ERR_CUDA;
  return CIL_OK;
}
