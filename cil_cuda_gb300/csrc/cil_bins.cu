// Rebuild of the binned element storage: a device counting sort that replaces the
// reference's linked-list cell grid (LinkListOrtho::populate_list, Utils.hpp:982-1001;
// LinkList/CellLinkList::populate, Container.cpp:58-103).
//
//   keys     one thread per used slot: bin id with the reference formula, atomic histogram
//   scan     per colony exclusive scan of the histogram -> range[b] = (first, end) slot
//   scatter  one thread per element: claim a slot inside its bin (atomic countdown, which
//            also returns the histogram to zero for the next rebuild)
//   sort     one thread per bin: order the bin's entries by element id (deterministic
//            result independent of the atomic order)
//   gather   one thread per destination slot: copy position, diameter, id; update slot_of;
//            write FP32 bin-local coordinates for the mixed-precision pair kernel
#include "cil_internal.cuh"

namespace cil {

namespace {

__device__ __forceinline__ int warp_incl_scan(int v) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) >= o) v += t;
  }
  return v;
}

// exclusive scan across a block of kTile threads; returns the exclusive prefix of v and
// the block total in *total
__device__ __forceinline__ int block_excl_scan(int v, int *total) {
  __shared__ int warp_sums[kTile / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int inc = warp_incl_scan(v);
  if (lane == 31) warp_sums[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    int w = lane < kTile / 32 ? warp_sums[lane] : 0;
    w = warp_incl_scan(w);
    if (lane < kTile / 32) warp_sums[lane] = w;
  }
  __syncthreads();
  const int base = wid > 0 ? warp_sums[wid - 1] : 0;
  *total = warp_sums[kTile / 32 - 1];
  __syncthreads();
  return base + inc - v;
}

// tiles[c] = sum over colonies < c of ceil(count_c / per); tiles[B] = total.
// which: 0 = nslot (per kTile), 1 = nlive (kTile), 2 = ncell (kCellTile), 3 = nslot in tiles of
// `per3` slots (slot pairs of the cell-major force kernel: twice its block size). A second table
// (which2, tiles2) can be written by the same launch.
__device__ __forceinline__ int tile_count(const ColonyCounters &k, int which, int per3) {
  const int n = which == 1 ? k.nlive : (which == 2 ? k.ncell : k.nslot);
  const int per = which == 2 ? kCellTile : (which == 3 ? per3 : kTile);
  return (n + per - 1) / per;
}

__global__ void k_tiles(const ColonyCounters *__restrict__ cnt, int B, int which, int *__restrict__ tiles,
                        int which2, int *__restrict__ tiles2, int per3) {
  int carry = 0, carry2 = 0;
  for (int base = 0; base < B; base += kTile) {
    const int c = base + threadIdx.x;
    const int v = c < B ? tile_count(cnt[c], which, per3) : 0;
    const int v2 = (tiles2 && c < B) ? tile_count(cnt[c], which2, per3) : 0;
    int total, total2;
    const int ex = block_excl_scan(v, &total);
    const int ex2 = block_excl_scan(v2, &total2);
    if (c < B) {
      tiles[c] = carry + ex;
      if (tiles2) tiles2[c] = carry2 + ex2;
    }
    carry += total;
    carry2 += total2;
  }
  if (threadIdx.x == 0) {
    tiles[B] = carry;
    if (tiles2) tiles2[B] = carry2;
  }
}

// New bin of a slot in the mixed form from FP32 data only: the home bin plus the whole
// bin widths its updated local coordinate has moved (periodic wrap; clamped along walls).
// shift[] receives the unwrapped change of the bin coordinate.
template <int D>
__device__ __forceinline__ void fast_bin(const ColonyConst &C, int home, const float4 &p, int *b, int *shift) {
  int h[D];
  bin_decode<D>(C, home, h);
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const int sh = static_cast<int>(floorf(pk_c(p, d) * C.inv_bwf[d]));
    int v = h[d] + sh;
    if (C.periodic[d]) {
      if (v < 0) v += C.ns[d];
      if (v >= C.ns[d]) v -= C.ns[d];
      shift[d] = sh;
    } else {
      v = v < 0 ? 0 : (v >= C.ns[d] ? C.ns[d] - 1 : v);
      shift[d] = v - h[d];
    }
    b[d] = v;
  }
}

template <int D>
__global__ void __launch_bounds__(kTile) k_bin_keys(RebuildArgs a) {
  const int total = a.tiles_used[a.B];
  for (int t = blockIdx.x; t < total; t += gridDim.x) {
    const int c = colony_of_tile(a.tiles_used, a.B, t);
    const ColonyConst &C = a.col[c];
    const int s = C.slot_base + (t - a.tiles_used[c]) * kTile + threadIdx.x;
    if (s >= C.slot_base + a.cnt[c].nslot) continue;
    int k = -1;
    if (a.eid_in[s] >= 0) {
      int b[D];
      if (a.exact) {
        double x[D];
#pragma unroll
        for (int d = 0; d < D; ++d) x[d] = a.x_in[d * a.SS + s];
        bin_coords<D>(C, x, b);
      } else {
        int sh[D];
        fast_bin<D>(C, a.sbin_in[s], a.pk_in[s], b, sh);
      }
      k = C.bin_base + bin_id<D>(C, b);
      atomicAdd(a.bcount + k, 1);
    }
    a.key[s] = k;
  }
}

// per scan block: sum of kScanItems bin counts
__device__ __forceinline__ bool skip_colony(const RebuildArgs &a, int c) {
  return a.skin != nullptr && !a.skin[c].rebuild_now;
}

// skin mode: no colony rebuilds this step (uniform over the grid; checked before any barrier)
__device__ __forceinline__ bool no_rebuild(const RebuildArgs &a) {
  return a.any_rebuild != nullptr && a.any_rebuild[*a.ts_dev & 1] == 0;
}

__global__ void __launch_bounds__(kTile) k_scan_partial(RebuildArgs a) {
  if (no_rebuild(a)) return;
  const int sb = blockIdx.x;
  if (skip_colony(a, a.scan_col[sb])) return;
  const ColonyConst &C = a.col[a.scan_col[sb]];
  const int b0 = C.bin_base + (sb - C.scan_base) * kScanItems;
  const int4 v = reinterpret_cast<const int4 *>(a.bcount + b0)[threadIdx.x];
  int s = v.x + v.y + v.z + v.w;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ int ws[kTile / 32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < kTile / 32; ++w) t += ws[w];
    a.scan_sum[sb] = t;
  }
}

// one block per colony: exclusive scan of its scan-block sums; nlive = nslot = total
__global__ void __launch_bounds__(kTile) k_scan_colony(RebuildArgs a) {
  if (no_rebuild(a)) return;
  const int c = blockIdx.x;
  if (skip_colony(a, c)) return;
  const ColonyConst &C = a.col[c];
  const int nsb = C.nbins_pad / kScanItems;
  int carry = 0;
  for (int base = 0; base < nsb; base += kTile) {
    const int i = base + threadIdx.x;
    const int v = i < nsb ? a.scan_sum[C.scan_base + i] : 0;
    int total;
    const int ex = block_excl_scan(v, &total);
    if (i < nsb) a.scan_off[C.scan_base + i] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0) {
    a.cnt[c].nlive = carry;
    if (a.permute) a.cnt[c].nslot = carry;
  }
}

// per scan block: bin ranges
__global__ void __launch_bounds__(kTile) k_scan_final(RebuildArgs a) {
  if (no_rebuild(a)) return;
  const int sb = blockIdx.x;
  if (skip_colony(a, a.scan_col[sb])) return;
  const ColonyConst &C = a.col[a.scan_col[sb]];
  const int b0 = C.bin_base + (sb - C.scan_base) * kScanItems + threadIdx.x * 4;
  const int4 v = *reinterpret_cast<const int4 *>(a.bcount + b0);
  const int sum = v.x + v.y + v.z + v.w;
  int total;
  const int ex = block_excl_scan(sum, &total);
  int start = C.slot_base + a.scan_off[sb] + ex;
  int2 *r = a.range + b0;
  r[0] = make_int2(start, start + v.x);
  start += v.x;
  r[1] = make_int2(start, start + v.y);
  start += v.y;
  r[2] = make_int2(start, start + v.z);
  start += v.z;
  r[3] = make_int2(start, start + v.w);
}

__global__ void __launch_bounds__(kTile) k_scatter(RebuildArgs a) {
  if (no_rebuild(a)) return;
  const int total = a.tiles_used[a.B];
  for (int t = blockIdx.x; t < total; t += gridDim.x) {
    const int c = colony_of_tile(a.tiles_used, a.B, t);
    if (skip_colony(a, c)) continue;
    const ColonyConst &C = a.col[c];
    const int s = C.slot_base + (t - a.tiles_used[c]) * kTile + threadIdx.x;
    // nslot was overwritten by the scan; the used-slot bound is the tile range itself and
    // every slot past the old nslot carries key -1 (k_clear_tail_keys / the rebin kernel).
    if (s >= C.slot_base + C.slot_cap) continue;
    const int k = a.key[s];
    if (k < 0) continue;
    const int pos = a.range[k].x + atomicSub(a.bcount + k, 1) - 1;
    a.perm[pos] = (static_cast<unsigned long long>(static_cast<uint32_t>(a.eid_in[s])) << 32) |
                  static_cast<uint32_t>(s);
  }
}

// Orders each bin's entries by element id. Bins hold a few elements: up to 8 are sorted in
// registers (insertion into a register array, then one coalesced write-back); larger bins
// fall back to an in-place insertion sort.
__global__ void __launch_bounds__(kTile) k_sort_bins(RebuildArgs a, int nbins_total) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nbins_total; b += gridDim.x * blockDim.x) {
    const int2 r = a.range[b];
    const int n = r.y - r.x;
    if (n < 2) continue;
    if (n <= 8) {
      unsigned long long v[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) v[i] = i < n ? a.perm[r.x + i] : ~0ull;
#pragma unroll
      for (int i = 1; i < 8; ++i)
#pragma unroll
        for (int k = i; k > 0; --k) {
          const unsigned long long lo = v[k - 1] < v[k] ? v[k - 1] : v[k];
          const unsigned long long hi = v[k - 1] < v[k] ? v[k] : v[k - 1];
          v[k - 1] = lo;
          v[k] = hi;
        }
#pragma unroll
      for (int i = 0; i < 8; ++i)
        if (i < n) a.perm[r.x + i] = v[i];
    } else {
      for (int i = r.x + 1; i < r.y; ++i) {
        const unsigned long long v = a.perm[i];
        int j = i - 1;
        while (j >= r.x && a.perm[j] > v) {
          a.perm[j + 1] = a.perm[j];
          --j;
        }
        a.perm[j + 1] = v;
      }
    }
  }
}

template <int D>
__global__ void __launch_bounds__(kTile) k_gather(RebuildArgs a) {
  const int total = a.tiles_live[a.B];
  for (int t = blockIdx.x; t < total; t += gridDim.x) {
    const int c = colony_of_tile(a.tiles_live, a.B, t);
    const ColonyConst &C = a.col[c];
    const int dst = C.slot_base + (t - a.tiles_live[c]) * kTile + threadIdx.x;
    if (dst >= C.slot_base + a.cnt[c].nlive) continue;
    const unsigned long long v = a.perm[dst];
    const int src = static_cast<int>(v & 0xffffffffu);
    const int e = static_cast<int>(v >> 32);
    const int g = e >> 1;
    double x[D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      x[d] = a.x_in[d * a.SS + src];
      a.x_out[d * a.SS + dst] = x[d];
    }
    if (a.vel_out) {
#pragma unroll
      for (int d = 0; d < D; ++d) a.vel_out[d * a.SS + dst] = a.vel_in[d * a.SS + src];
    }
    a.eid_out[dst] = e;
    a.slot_of[e] = dst;
    if (a.state_out) {
      // skin mode: the new order is the bin order, so a bin's members are its own slots
      a.state_out[dst] = kSlotNormal;
      a.perm[dst] = (static_cast<unsigned long long>(static_cast<uint32_t>(e)) << 32) | static_cast<uint32_t>(dst);
    }
    const int nb = a.key[src] - C.bin_base;  // colony-local bin of the element
    a.sbin_out[dst] = nb;
    if (a.exact) {
      a.cyc_out[dst] = make_int2(a.t0c[g], a.tswc[g]);
      const double sg = a.sigma_c[e];
      if (a.sig_out) a.sig_out[dst] = sg;
      if (a.pk_out) {
        int b[D];
        bin_decode<D>(C, nb, b);
        float4 p = make_float4(0.0f, 0.0f, 0.0f, static_cast<float>(sg));
#pragma unroll
        for (int d = 0; d < D; ++d) pk_set(p, d, static_cast<float>(x[d] - static_cast<double>(b[d]) * C.bw[d]));
        a.pk_out[dst] = p;
      }
    } else {
      a.cyc_out[dst] = a.cyc_in[src];
      if (a.sig_out) a.sig_out[dst] = a.sig_in[src];
      if (a.pk_out) {
        int b[D], sh[D];
        const float4 q = a.pk_in[src];
        fast_bin<D>(C, a.sbin_in[src], q, b, sh);
        float4 p = make_float4(0.0f, 0.0f, 0.0f, fabsf(q.w));  // every element is normal after a re-sort
#pragma unroll
        for (int d = 0; d < D; ++d) pk_set(p, d, pk_c(q, d) - static_cast<float>(sh[d]) * C.bwf[d]);
        a.pk_out[dst] = p;
      }
    }
  }
}

// marks the slots past the used range as empty so that the scatter pass sees key -1
__global__ void __launch_bounds__(kTile) k_clear_tail_keys(RebuildArgs a) {
  const int c = blockIdx.y;
  const ColonyConst &C = a.col[c];
  const int used = a.cnt[c].nslot;
  for (int i = used + blockIdx.x * blockDim.x + threadIdx.x; i < ((used + kTile - 1) / kTile) * kTile;
       i += gridDim.x * blockDim.x)
    if (i < C.slot_cap) a.key[C.slot_base + i] = -1;
}

// ---------------------------------------------------------------- cell-major slot re-sort
// Skin mode re-sorts its slots by cell: cells are ranked by the bin of their back element (a
// counting sort over the same bins and scan kernels), and the two elements of the cell of rank
// r move into the slot pair (slot_base + 2 r, + 1), back element first. Tombstones are dropped
// (nslot = 2 ncell). Each element keeps its own home bin, so the Verlet lists (built next from
// the element bins) do not depend on the slot order; only the force kernel, one thread per slot
// pair, does.

// cell c-local index i of thread (tile t, item q) over tiles_cell
__device__ __forceinline__ int cell_of(const RebuildArgs &a, int t, int c, int q) {
  return (t - a.tiles_cell[c]) * kCellTile + q * kTile + threadIdx.x;
}

template <int D>
__device__ __forceinline__ int cell_bin(const RebuildArgs &a, const ColonyConst &C, int s) {
  int b[D];
  if (a.exact) {
    double x[D];
#pragma unroll
    for (int d = 0; d < D; ++d) x[d] = a.x_in[d * a.SS + s];
    bin_coords<D>(C, x, b);
  } else {
    int sh[D];
    fast_bin<D>(C, a.sbin_in[s], a.pk_in[s], b, sh);
  }
  return bin_id<D>(C, b);
}

template <int D>
__global__ void __launch_bounds__(kTile) k_cell_keys(RebuildArgs a) {
  const int total = a.tiles_cell[a.B];
  for (int t = blockIdx.x; t < total; t += gridDim.x) {
    const int c = colony_of_tile(a.tiles_cell, a.B, t);
    const ColonyConst &C = a.col[c];
    const int n = a.cnt[c].ncell;
#pragma unroll
    for (int q = 0; q < kCellItems; ++q) {
      const int i = cell_of(a, t, c, q);
      if (i >= n) continue;
      const int g = C.cell_base + i;
      const int k = C.bin_base + cell_bin<D>(a, C, a.slot_of[2 * g]);
      a.key[g] = k;
      atomicAdd(a.bcount + k, 1);
    }
  }
}

// rank of every cell inside its bin's range (bcount counts back down to zero); perm[slot_base
// + rank] = cell
__global__ void __launch_bounds__(kTile) k_cell_scatter(RebuildArgs a) {
  const int total = a.tiles_cell[a.B];
  for (int t = blockIdx.x; t < total; t += gridDim.x) {
    const int c = colony_of_tile(a.tiles_cell, a.B, t);
    const ColonyConst &C = a.col[c];
    const int n = a.cnt[c].ncell;
#pragma unroll
    for (int q = 0; q < kCellItems; ++q) {
      const int i = cell_of(a, t, c, q);
      if (i >= n) continue;
      const int g = C.cell_base + i;
      const int k = a.key[g];
      const int pos = a.range[k].x + atomicSub(a.bcount + k, 1) - 1;  // slot_base + rank
      a.perm[pos] = static_cast<unsigned long long>(static_cast<uint32_t>(g));
    }
  }
}

template <int D>
__global__ void __launch_bounds__(kTile) k_cell_gather(RebuildArgs a) {
  const int total = a.tiles_cell[a.B];
  for (int t = blockIdx.x; t < total; t += gridDim.x) {
    const int c = colony_of_tile(a.tiles_cell, a.B, t);
    const ColonyConst &C = a.col[c];
    const int n = a.cnt[c].ncell;
#pragma unroll
    for (int q = 0; q < kCellItems; ++q) {
      const int r = cell_of(a, t, c, q);
      if (r >= n) continue;
      const int g = static_cast<int>(a.perm[C.slot_base + r] & 0xffffffffu);
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int e = 2 * g + j;
        const int src = a.slot_of[e];
        const int dst = C.slot_base + 2 * r + j;
        double x[D];
#pragma unroll
        for (int d = 0; d < D; ++d) {
          x[d] = a.x_in[d * a.SS + src];
          a.x_out[d * a.SS + dst] = x[d];
        }
        if (a.vel_out) {
#pragma unroll
          for (int d = 0; d < D; ++d) a.vel_out[d * a.SS + dst] = a.vel_in[d * a.SS + src];
        }
        a.eid_out[dst] = e;
        a.slot_of[e] = dst;
        a.state_out[dst] = kSlotNormal;
        if (a.sig_out) a.sig_out[dst] = a.sig_in[src];
        int b[D];
        float4 p;
        if (a.exact) {
          // re-anchored on the FP64 position: home bin and local coordinate from x
          a.cyc_out[dst] = make_int2(a.t0c[g], a.tswc[g]);
          bin_coords<D>(C, x, b);
          p = make_float4(0.0f, 0.0f, 0.0f, static_cast<float>(a.sigma_c[e]));
#pragma unroll
          for (int d = 0; d < D; ++d) pk_set(p, d, static_cast<float>(x[d] - static_cast<double>(b[d]) * C.bw[d]));
        } else {
          a.cyc_out[dst] = a.cyc_in[src];
          int sh[D];
          const float4 qv = a.pk_in[src];
          fast_bin<D>(C, a.sbin_in[src], qv, b, sh);
          p = make_float4(0.0f, 0.0f, 0.0f, fabsf(qv.w));  // every element is normal after a re-sort
#pragma unroll
          for (int d = 0; d < D; ++d) pk_set(p, d, pk_c(qv, d) - static_cast<float>(sh[d]) * C.bwf[d]);
        }
        a.pk_out[dst] = p;
        a.sbin_out[dst] = bin_id<D>(C, b);
      }
    }
  }
}

// per colony: the slot pairs in use after the re-sort
__global__ void k_cell_finish(RebuildArgs a) {
  for (int c = threadIdx.x; c < a.B; c += blockDim.x) a.cnt[c].nslot = 2 * a.cnt[c].ncell;
}

}  // namespace

void launch_tiles(const ColonyConst *, ColonyCounters *cnt, int B, int which, int *tiles,
                  cudaStream_t s, int which2, int *tiles2, int per2) {
  k_tiles<<<1, kTile, 0, s>>>(cnt, B, which, tiles, which2, tiles2, per2);
}

void launch_rebuild(const RebuildArgs &a, int grid_slots, cudaStream_t s) {
  // keys + histogram over the used slots (tiles_used must be current); a non-permuting
  // rebuild (skin mode) gets its keys from the in-place rebin kernel instead
  if (a.permute) {
    k_clear_tail_keys<<<dim3(1, a.B), kTile, 0, s>>>(a);
    if (a.dim == 2)
      k_bin_keys<2><<<grid_slots, kTile, 0, s>>>(a);
    else
      k_bin_keys<3><<<grid_slots, kTile, 0, s>>>(a);
  }
  k_scan_partial<<<a.nscan, kTile, 0, s>>>(a);
  k_scan_colony<<<a.B, kTile, 0, s>>>(a);
  k_scan_final<<<a.nscan, kTile, 0, s>>>(a);
  k_scatter<<<grid_slots, kTile, 0, s>>>(a);
  if (!a.permute) return;  // the bin index (range + perm) is all a list rebuild needs
  if (a.skin == nullptr)   // bin order by element id: deterministic sums (FP64 / plain forms)
    k_sort_bins<<<(a.nscan * kScanItems + kTile - 1) / kTile, kTile, 0, s>>>(a, a.nscan * kScanItems);
  k_tiles<<<1, kTile, 0, s>>>(a.cnt, a.B, 1, const_cast<int *>(a.tiles_live), 0, nullptr, 2 * kTile);
  if (a.dim == 2)
    k_gather<2><<<grid_slots, kTile, 0, s>>>(a);
  else
    k_gather<3><<<grid_slots, kTile, 0, s>>>(a);
}

void launch_cell_resort(const RebuildArgs &a, int grid_cells, cudaStream_t s) {
  if (a.dim == 2)
    k_cell_keys<2><<<grid_cells, kTile, 0, s>>>(a);
  else
    k_cell_keys<3><<<grid_cells, kTile, 0, s>>>(a);
  k_scan_partial<<<a.nscan, kTile, 0, s>>>(a);
  k_scan_colony<<<a.B, kTile, 0, s>>>(a);
  k_scan_final<<<a.nscan, kTile, 0, s>>>(a);
  k_cell_scatter<<<grid_cells, kTile, 0, s>>>(a);
  if (a.dim == 2)
    k_cell_gather<2><<<grid_cells, kTile, 0, s>>>(a);
  else
    k_cell_gather<3><<<grid_cells, kTile, 0, s>>>(a);
  k_cell_finish<<<1, kTile, 0, s>>>(a);
}

}  // namespace cil
