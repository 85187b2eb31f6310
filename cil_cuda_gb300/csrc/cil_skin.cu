// Verlet-skin mode of the mixed-precision step.
//
// The reference rebuilds its link list every step (CIL.cu:180); with a skin the bins and
// per-element Verlet lists (cutoff rc_ij + skin) are kept for as long as every element stays
// within skin/2 of its position at the last build (the displacement guard, checked by the
// force kernel every step), or until the cadence chosen for the colony expires.
//
//   k_skin_begin   per colony: turn the guard / cadence / host requests into rebuild_now
//   k_skin_rebin   rebuilding colonies: new home bin of every slot from its FP32 local
//                  coordinate (in place, no data movement) and the bin histogram
//   (scan + scatter of cil_bins.cu give range[] and perm[] for the rebuilding colonies)
//   k_skin_lists   rebuilding colonies: Verlet list of every live slot from the 3^d bins;
//                  entries are slot | (neighbour-bin index << 27); same-cell elements are
//                  excluded; uref = u; every slot becomes "normal"
//   k_fresh_pairs  elements created or moved by a division since the last build ("fresh")
//                  are in no list: each searches the bins of the last build for normal
//                  partners (Newton's third law onto them through facc) and the per-bin
//                  fresh lists for fresh partners; normal elements skip fresh candidates
//                  in their lists
#include "cil_internal.cuh"

namespace cil {
namespace {

template <int D>
__device__ __forceinline__ void nb_offsets(int o, int *off) {
  if (D == 2) {
    off[0] = o / 3 - 1;
    off[1] = o % 3 - 1;
  } else {
    off[0] = o / 9 - 1;
    off[1] = (o / 3) % 3 - 1;
    off[2] = o % 3 - 1;
  }
}

template <int D>
__device__ __forceinline__ bool nb_bin(const ColonyConst &C, const int *bi, const int *o, int *nb) {
#pragma unroll
  for (int d = 0; d < D; ++d) {
    int v = bi[d] + o[d];
    if (v < 0) {
      if (!C.periodic[d]) return false;
      v += C.ns[d];
    } else if (v >= C.ns[d]) {
      if (!C.periodic[d]) return false;
      v -= C.ns[d];
    }
    nb[d] = v;
  }
  return true;
}

__device__ __forceinline__ float log_disp(float d) { return 0.25f * log10f(fmaxf(d, 1e-8f)) + 1.0f; }

// per colony (lane 0 of the colony's warp): the rebuild decision and, at a rebuild, the
// scheduler's features; returns whether the colony rebuilds this step
__device__ __forceinline__ int skin_begin_colony(const SkinArgs &a, int c) {
  ColonySkin &S = a.skin[c];
  int need = S.need;
  if (a.force_rebuild) need |= 8;
  if (S.interval > 0 && S.steps_since >= S.interval) need |= 4;
  const int now = need != 0 ? 1 : 0;
  S.rebuild_now = now;
  SchedState &Q = a.sched[c];
  const ColonyCounters &K = a.cnt[c];
  const float n = fmaxf(static_cast<float>(K.ncell), 1.0f);
  {
    // event rates per cell per step, moving averages over ~100 steps
    const float dr = static_cast<float>(K.ndiv_total - Q.ndiv_prev) / n;
    const float ar = static_cast<float>(K.napo_total - Q.napo_prev) / n;
    Q.ndiv_prev = K.ndiv_total;
    Q.napo_prev = K.napo_total;
    Q.div_rate = 0.99f * Q.div_rate + 0.01f * dr;
    Q.apo_rate = 0.99f * Q.apo_rate + 0.01f * ar;
  }
  if (now) {
    // features of the decision taken at this rebuild:
    //   0 log(cells)/14              1 mean home-bin occupancy/10   2 max bin occupancy/20
    //   3 mean step displacement     4 max step displacement (both log10/4 + 1)
    //   5 divisions /cell/step x1e4  6 apoptoses /cell/step x1e4
    //   7 current skin               8 log(1 + steps since the last rebuild)/5
    //   9 largest displacement from the list reference / (skin/2)
    //   10 share of guard-triggered rebuilds   11 fresh elements / elements x10
    const float ne = 2.0f * n;
    const float disp = sqrtf(__uint_as_float(S.maxdisp2));
    const float occn = fmaxf(static_cast<float>(Q.occ_count), 1.0f);
    float *x = Q.features;
    x[0] = logf(n) / 14.0f;
    x[1] = Q.occ_sum / occn / 10.0f;
    x[2] = Q.occ_max / 20.0f;
    x[3] = log_disp(Q.step_sum / ne);
    x[4] = log_disp(Q.step_max);
    x[5] = Q.div_rate * 1e4f;
    x[6] = Q.apo_rate * 1e4f;
    x[7] = S.skin;
    x[8] = log1pf(static_cast<float>(S.steps_since)) / 5.0f;
    x[9] = S.skin > 0.0f ? disp / (0.5f * S.skin) : 0.0f;
    Q.trip_share = 0.9f * Q.trip_share + ((need & 1) ? 0.1f : 0.0f);
    x[10] = Q.trip_share;
    x[11] = 10.0f * static_cast<float>(S.nfresh) / ne;
    Q.occ_sum = 0.0f;
    Q.occ_max = 0.0f;
    Q.occ_count = 0;
    if (need & 1) S.ntrip += 1;
    S.last_interval = S.steps_since;
    S.steps_since = 0;
    S.nrebuild += 1;
    S.nfresh = 0;
    S.npairs = 0;
    S.list_overflow = 0;
    S.need = 0;
  }
  Q.step_sum = 0.0f;
  Q.step_max = 0.0f;
  S.steps_since += 1;
  S.maxdisp2 = 0u;
  return now;
}

// one warp per colony: the decision, then (rebuilding colony, scheduler installed) the
// network on the colony's features sets the skin of the new lists and the cadence
__global__ void k_skin_begin(SkinArgs a) {
  if (blockIdx.x == 0 && a.tiles_used_out) {
    // the step's tile tables (slots: kTile per tile; slot pairs: pair_tile slots per tile),
    // block 0, before any thread returns
    __shared__ int ws[2][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int carry0 = 0, carry1 = 0;
    for (int base = 0; base < a.B; base += blockDim.x) {
      const int cc = base + static_cast<int>(threadIdx.x);
      const int ns = cc < a.B ? a.cnt[cc].nslot : 0;
      int v[2] = {(ns + kTile - 1) / kTile, (ns + a.pair_tile - 1) / a.pair_tile};
      int inc[2] = {v[0], v[1]};
#pragma unroll
      for (int o = 1; o < 32; o <<= 1)
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const int t = __shfl_up_sync(0xffffffffu, inc[q], o);
          if (lane >= o) inc[q] += t;
        }
      if (lane == 31) {
        ws[0][wid] = inc[0];
        ws[1][wid] = inc[1];
      }
      __syncthreads();
      int before[2] = {0, 0}, tot[2] = {0, 0};
      for (int w = 0; w < nw; ++w)
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          before[q] += w < wid ? ws[q][w] : 0;
          tot[q] += ws[q][w];
        }
      if (cc < a.B) {
        a.tiles_used_out[cc] = carry0 + before[0] + inc[0] - v[0];
        a.tiles_pairs_out[cc] = carry1 + before[1] + inc[1] - v[1];
      }
      carry0 += tot[0];
      carry1 += tot[1];
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      a.tiles_used_out[a.B] = carry0;
      a.tiles_pairs_out[a.B] = carry1;
    }
  }
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (c >= a.B) return;  // uniform per warp
  const int lane = threadIdx.x & 31;
  int now = 0;
  {
    // the last force pass's displacement statistics, folded from the colony's slots
    StatPart &P = a.spart[c * kStatSlots + lane];
    const unsigned dmax = __reduce_max_sync(0xffffffffu, P.dmax);
    const unsigned smax = __reduce_max_sync(0xffffffffu, P.smax);
    float ssum = P.ssum;
#pragma unroll
    for (int q = 16; q > 0; q >>= 1) ssum += __shfl_xor_sync(0xffffffffu, ssum, q);
    P.dmax = 0u;
    P.smax = 0u;
    P.ssum = 0.0f;
    if (lane == 0) {
      a.skin[c].maxdisp2 = dmax;
      a.sched[c].step_max = __uint_as_float(smax);
      a.sched[c].step_sum = ssum;
    }
  }
  if (lane == 0) {
    now = skin_begin_colony(a, c);
    if (now && a.any_rebuild) atomicOr(&a.any_rebuild[*a.ts_dev & 1], 1);
    if (a.use_cond) {
      // the last colony to decide sets the step's rebuild node (one caller: no racing sets)
      __threadfence();
      if (atomicAdd(&a.any_rebuild[2], 1) == a.B - 1) {
        __threadfence();
        const int any = atomicOr(&a.any_rebuild[*a.ts_dev & 1], 0);
        cudaGraphSetConditional(a.cond, any != 0 ? 1u : 0u);
        if (any) atomicAdd(&a.any_rebuild[3], 1);
        atomicExch(&a.any_rebuild[2], 0);
      }
    }
  }
  now = __shfl_sync(0xffffffffu, now, 0);
  if (!now || !a.mlp) return;  // uniform per warp
  __syncwarp();
  SchedState &Q = a.sched[c];
  float x[kMlpIn];
#pragma unroll
  for (int k = 0; k < kMlpIn; ++k) x[k] = Q.features[k];
  float y[kMlpOut];
  mlp_forward_warp(a.mlp, x, y);
  if (lane == 0) {
    ColonySkin &S = a.skin[c];
    const float sg = 1.0f / (1.0f + expf(-y[0]));
    const float skin = a.skin_min + (a.skin_max - a.skin_min) * sg;
    const float sp = y[1] > 20.0f ? y[1] : log1pf(expf(y[1]));
    int interval = static_cast<int>(fminf(rintf(a.interval_scale * sp), 1e6f));
    interval = interval < 1 ? 1 : interval;
    S.skin = skin;
    S.half2 = 0.25f * skin * skin;
    S.interval = a.use_interval ? interval : 0;
    Q.nsched += 1;
  }
}

template <int D>
__global__ void __launch_bounds__(kTile) k_skin_rebin(SkinArgs a) {
  if (a.any_rebuild && a.any_rebuild[*a.ts_dev & 1] == 0) return;  // uniform
  const int total = a.tiles[a.B];
  for (int t = blockIdx.x; t < total; t += gridDim.x) {
    const int c = colony_of_tile(a.tiles, a.B, t);
    if (!a.skin[c].rebuild_now) continue;
    const ColonyConst &C = a.col[c];
    const int s = C.slot_base + (t - a.tiles[c]) * kTile + threadIdx.x;
    int k = -1;
    if (s < C.slot_base + a.cnt[c].nslot && a.eid[s] >= 0 && a.state[s] != kSlotDead) {
      int h[D], b[D];
      bin_decode<D>(C, a.sbin[s], h);
      float4 p = a.pk[s];
#pragma unroll
      for (int d = 0; d < D; ++d) {
        float u = pk_c(p, d);
        const int sh = static_cast<int>(floorf(u * C.inv_bwf[d]));
        int v = h[d] + sh;
        if (C.periodic[d]) {
          if (v < 0) v += C.ns[d];
          if (v >= C.ns[d]) v -= C.ns[d];
          u -= static_cast<float>(sh) * C.bwf[d];
        } else {
          const int vc = v < 0 ? 0 : (v >= C.ns[d] ? C.ns[d] - 1 : v);
          u -= static_cast<float>(vc - h[d]) * C.bwf[d];
          v = vc;
        }
        b[d] = v;
        pk_set(p, d, u);
      }
      a.pk[s] = p;
      const int id = bin_id<D>(C, b);
      a.sbin[s] = id;
      k = C.bin_base + id;
      atomicAdd(a.bcount + k, 1);
    }
    if (s < C.slot_base + C.slot_cap) a.key[s] = k;
  }
}

// Latency-bound (two dependent loads per batch of candidates): many resident warps with short
// batches beat few warps with long ones. One list build (with the rebin and scan launches) of
// the 2M-particle 2D colony took 0.603 ms with batches of 8 at 2 CTAs per SM (108 registers),
// 0.440 ms with 4 at 4 CTAs and 0.420 ms with 2 at 8 CTAs (32 registers); of the 4M-particle
// 3D channel, 2.64 ms with 8 at 1 CTA, 1.55 ms with 2 at 2 CTAs and 1.43 ms with 2 at 3 CTAs
// (3D keeps the 27 bin ranges in registers, so it runs fewer CTAs per SM).
template <int D>
constexpr int kListBatch = 2;
template <int D>
constexpr int kListMinBlocks = D == 2 ? 8 : 3;

template <int D, int LAW>
__global__ void __launch_bounds__(kTile, kListMinBlocks<D>) k_skin_lists(SkinArgs a) {
  constexpr int NB = (D == 2) ? 9 : 27;
  if (a.any_rebuild && a.any_rebuild[*a.ts_dev & 1] == 0) return;  // uniform, before any barrier
  __shared__ unsigned s_occ_sum, s_occ_max, s_cnt;
  __shared__ unsigned long long s_pairs;
  __shared__ int s_over;
  const int total = a.tiles[a.B];
  for (int t = blockIdx.x; t < total; t += gridDim.x) {
    const int c = colony_of_tile(a.tiles, a.B, t);
    ColonySkin &S = a.skin[c];
    if (!S.rebuild_now) continue;  // uniform per block
    if (threadIdx.x == 0) {
      s_occ_sum = 0u;
      s_occ_max = 0u;
      s_cnt = 0u;
      s_pairs = 0ull;
      s_over = 0;
    }
    __syncthreads();
    const ColonyConst &C = a.col[c];
    const int s = C.slot_base + (t - a.tiles[c]) * kTile + threadIdx.x;
    const size_t SS = a.SS;
    int n = 0;
    unsigned occ = 0u, counted = 0u;
    if (s < C.slot_base + a.cnt[c].nslot) {
      const int e = a.eid[s];
      if (e < 0 || a.state[s] == kSlotDead) {
        a.ncnt[s] = 0;
      } else {
        const int g = e >> 1;
        float4 pi = a.pk[s];
        float ui[D];
#pragma unroll
        for (int d = 0; d < D; ++d) ui[d] = pk_c(pi, d);
        const float si = fabsf(pi.w);
        const float skin = S.skin;
        int bi[D];
        bin_decode<D>(C, a.sbin[s], bi);
        // the 3^d bin ranges, loaded together; candidates are then taken as one flattened
        // range in batches of kLB, so each batch costs two round trips (slots, then records)
        constexpr int kLB = kListBatch<D>;
        int start[NB], pre[NB + 1];
        pre[0] = 0;
#pragma unroll
        for (int o = 0; o < NB; ++o) {
          int off[3];
          nb_offsets<D>(o, off);
          int nb[D];
          int2 r = make_int2(0, 0);
          if (nb_bin<D>(C, bi, off, nb)) r = a.range[C.bin_base + bin_id<D>(C, nb)];
          start[o] = r.x;
          pre[o + 1] = pre[o] + (r.y - r.x);
          if (o == NB / 2) occ = static_cast<unsigned>(r.y - r.x);  // the home bin
        }
        const int ncand = pre[NB];
        for (int k0 = 0; k0 < ncand; k0 += kLB) {
          int tt[kLB], oo[kLB];
#pragma unroll
          for (int q = 0; q < kLB; ++q) {
            const int kq = k0 + q;
            int o = 0, base = start[0];  // select chain: constant indices keep the arrays in registers
#pragma unroll
            for (int b = 1; b < NB; ++b) {
              if (kq >= pre[b]) {
                o = b;
                base = start[b] - pre[b];
              }
            }
            oo[q] = o;
            tt[q] = kq < ncand ? static_cast<int>(a.perm[base + kq] & 0xffffffffu) : -1;
          }
          int ej[kLB];
          float4 pj[kLB];
#pragma unroll
          for (int q = 0; q < kLB; ++q) {
            ej[q] = tt[q] >= 0 ? a.eid[tt[q]] : -2;
            pj[q] = tt[q] >= 0 ? a.pk[tt[q]] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
          }
#pragma unroll
          for (int q = 0; q < kLB; ++q) {
            if (tt[q] < 0 || tt[q] == s || (ej[q] >> 1) == g) continue;
            int off[3];
            nb_offsets<D>(oo[q], off);
            float r2 = 0.0f;
#pragma unroll
            for (int d = 0; d < D; ++d) {
              const float dx = pk_c(pj[q], d) + (static_cast<float>(off[d]) * C.bwf[d] - ui[d]);
              r2 += dx * dx;
            }
            const float cut = law_cutoff_f<LAW>(C, si, fabsf(pj[q].w)) + skin;
            if (r2 < cut * cut) {
              if (n < kListCap)
                a.nbr[static_cast<size_t>(n) * SS + s] =
                    tt[q] | static_cast<int>(list_offset_code(oo[q], D) << kListSlotBits);
              ++n;
            }
          }
        }
        a.ncnt[s] = n < kListCap ? n : kListCap;
        if (D == 2) {
          a.pk[s].z = uref_pack2(C.uq_scale, ui[0], ui[1]);  // list reference in the record
        } else {
#pragma unroll
          for (int d = 0; d < D; ++d) a.uref[d * SS + s] = ui[d];
        }
        a.state[s] = kSlotNormal;
        counted = 1u;
        a.pk[s].w = si;  // normal: visible to the lists of others
      }
    }
    // list and scheduler statistics: warp reductions, shared atomics, one global atomic each
    const unsigned w_sum = __reduce_add_sync(0xffffffffu, occ);
    const unsigned w_max = __reduce_max_sync(0xffffffffu, occ);
    const unsigned w_cnt = __reduce_add_sync(0xffffffffu, counted);
    const unsigned w_pairs = __reduce_add_sync(0xffffffffu, static_cast<unsigned>(n));
    const unsigned w_over = __reduce_add_sync(0xffffffffu, n > kListCap ? 1u : 0u);
    if ((threadIdx.x & 31) == 0) {
      atomicAdd(&s_occ_sum, w_sum);
      atomicMax(&s_occ_max, w_max);
      atomicAdd(&s_cnt, w_cnt);
      atomicAdd(&s_pairs, static_cast<unsigned long long>(w_pairs));
      atomicAdd(&s_over, static_cast<int>(w_over));
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      SchedState &Q = a.sched[c];
      atomicAdd(&Q.occ_sum, static_cast<float>(s_occ_sum));
      atomicAdd(&Q.occ_count, static_cast<int>(s_cnt));
      atomicMax(reinterpret_cast<unsigned *>(&Q.occ_max), __float_as_uint(static_cast<float>(s_occ_max)));
      atomicAdd(reinterpret_cast<unsigned long long *>(&S.npairs), s_pairs);
      if (s_over) {
        atomicAdd(&S.list_overflow, s_over);
        atomicOr(&a.cnt[c].err, kErrCap);
      }
    }
    __syncthreads();
  }
}

// After a list build, the lists of each warp of the force kernel (32 cells = 64 slots from a
// 64-aligned first slot w0) as one contiguous range in the warp's flattened order (element by
// element, each list in order) at w0 * kListCap, with the owner (element of the warp) of every
// entry, each element's start in the range (lstart) and the warp's entry count (lwarp): the force
// kernel then copies a warp's entries and owners with a few 16-byte copies per lane. One block of
// 128 threads per tile of kTile slots (4 warps of 64 slots), rebuilding colonies only; each warp
// assembles segments of kFlatSeg entries in shared memory and stores them with 16-byte stores.
constexpr int kFlatSeg = 1024;

__global__ void __launch_bounds__(128) k_list_flatten(SkinArgs a) {
  __shared__ __align__(16) int s_ent[4][kFlatSeg];
  __shared__ __align__(16) unsigned char s_own[4][kFlatSeg];
  const int total = a.tiles[a.B];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int t = blockIdx.x; t < total; t += gridDim.x) {
    const int c = colony_of_tile(a.tiles, a.B, t);
    if (!a.skin[c].rebuild_now) continue;  // uniform per block
    const ColonyConst &C = a.col[c];
    const int s0 = C.slot_base + (t - a.tiles[c]) * kTile + 2 * threadIdx.x;
    const int nslot = a.cnt[c].nslot;
    const int2 n = s0 < C.slot_base + nslot ? *reinterpret_cast<const int2 *>(a.ncnt + s0) : make_int2(0, 0);
    const int cnt = n.x + n.y;
    int inc = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += v;
    }
    const int T = __shfl_sync(0xffffffffu, inc, 31);
    const int st0 = inc - cnt, st1 = st0 + n.x;
    const int w0 = s0 - 2 * lane;
    if (s0 < C.slot_base + C.slot_cap)
      *reinterpret_cast<ushort2 *>(a.lstart + s0) =
          make_ushort2(static_cast<unsigned short>(st0), static_cast<unsigned short>(st1));
    if (lane == 31) a.lwarp[w0 >> 6] = inc;
    if (t == a.tiles[c] && threadIdx.x == 0) a.skin[c].nslot_built = nslot;
    int *dst = a.lflat + static_cast<size_t>(w0) * kListCap;
    unsigned char *dso = a.oflat + static_cast<size_t>(w0) * kListCap;
    int *se = s_ent[wid];
    unsigned char *so = s_own[wid];
    for (int S = 0; S < T; S += kFlatSeg) {  // uniform per warp
      const int E = min(T, S + kFlatSeg);
      // this lane's entries of the segment, read row by row (the list rows are SS apart)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int st = j ? st1 : st0, nj = j ? n.y : n.x;
        const int k0 = max(S - st, 0), k1 = min(E - st, nj);
        for (int k = k0; k < k1; k += 4) {
          int v[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) v[q] = k + q < k1 ? __ldg(a.nbr + static_cast<size_t>(k + q) * a.SS + s0 + j) : 0;
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            if (k + q < k1) {
              se[st + k + q - S] = v[q];
              so[st + k + q - S] = static_cast<unsigned char>(2 * lane + j);
            }
          }
        }
      }
      __syncwarp();
      // 16-byte stores of the segment (rounded up to 4 entries / 16 owners: within the warp's
      // 64 kListCap entries and within the shared segment)
      const int ne = (E - S + 3) >> 2, no = (E - S + 15) >> 4;
      for (int i = lane; i < ne; i += 32)
        *reinterpret_cast<int4 *>(dst + S + 4 * i) = *reinterpret_cast<const int4 *>(se + 4 * i);
      for (int i = lane; i < no; i += 32)
        *reinterpret_cast<int4 *>(dso + S + 16 * i) = *reinterpret_cast<const int4 *>(so + 16 * i);
      __syncwarp();
    }
  }
}

// Fresh elements (created or moved by divisions since the last build) against the normal
// elements in the bins of the last build (with Newton's third law onto them through facc)
// and against the other fresh elements through the per-bin fresh lists. One warp per fresh
// element: the lanes take the 3^d bins' candidates as one flattened range, so the loads of
// all candidates are in flight together.
constexpr int kFreshBlock = 128, kFreshWarps = kFreshBlock / 32;

template <int D, int LAW>
__global__ void __launch_bounds__(kFreshBlock) k_fresh_pairs(SkinArgs a) {
  constexpr int NB = (D == 2) ? 9 : 27;
  // the fresh sets of all colonies as one flattened range (inclusive prefix of their sizes)
  extern __shared__ int s_pref[];  // [B], sized at launch (all blocks resident in one wave)
  __shared__ int s_warp[kFreshWarps];
  __shared__ int s_run;
  const int nb_col = a.B;  // <= kMaxSkinColonies (checked at create)
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_run = 0;
  __syncthreads();
  for (int c0 = 0; c0 < nb_col; c0 += kFreshBlock) {
    const int c = c0 + threadIdx.x;
    int v = c < nb_col ? min(a.skin[c].nfresh, kFreshCap) : 0;
#pragma unroll
    for (int q = 1; q < 32; q <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, v, q);
      if (lane >= q) v += u;
    }
    if (lane == 31) s_warp[wid] = v;
    __syncthreads();
    int base = s_run;
    for (int w = 0; w < wid; ++w) base += s_warp[w];
    if (c < nb_col) s_pref[c] = base + v;
    __syncthreads();
    if (threadIdx.x == kFreshBlock - 1) s_run = base + v;
    __syncthreads();
  }
  const int total_fresh = s_run;
  for (int gi = blockIdx.x * kFreshWarps + (threadIdx.x >> 5); gi < total_fresh; gi += gridDim.x * kFreshWarps) {
    int lo = 0, hi = nb_col - 1;  // colony: first with s_pref > gi
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (s_pref[mid] > gi)
        hi = mid;
      else
        lo = mid + 1;
    }
    const int c = lo;
    const int i = gi - (c > 0 ? s_pref[c - 1] : 0);
    const ColonySkin &S = a.skin[c];
    const unsigned epoch = static_cast<unsigned>(S.nrebuild);
    const ColonyConst &C = a.col[c];
    const size_t SS = a.SS;
    const float eps = C.eps_f, rcs = C.rcs_f;
    const int f = a.fresh[c * kFreshCap + i];
    if (a.state[f] != kSlotFresh || a.eid[f] < 0) continue;  // uniform per warp
    const int gf = a.eid[f] >> 1;
    const float4 pf = a.pk[f];
    const float sf = fabsf(pf.w);
    int bf[D];
    bin_decode<D>(C, a.sbin[f], bf);
    // lane o < NB: neighbour bin o (offset, range)
    int bin = -1, cnt = 0;
    float ofs[3] = {0.0f, 0.0f, 0.0f};
    if (lane < NB) {
      int off[3];
      nb_offsets<D>(lane, off);
      int nb[D];
      if (nb_bin<D>(C, bf, off, nb)) {
        bin = C.bin_base + bin_id<D>(C, nb);
        const int2 r = a.range[bin];
        cnt = r.y - r.x;
#pragma unroll
        for (int d = 0; d < D; ++d) ofs[d] = static_cast<float>(off[d]) * C.bwf[d] - pk_c(pf, d);
      }
    }
    int incl = cnt;
#pragma unroll
    for (int q = 1; q < 32; q <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, q);
      if (lane >= q) incl += v;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const int start = (bin >= 0) ? a.range[bin].x : 0;
    float acc[D];
#pragma unroll
    for (int d = 0; d < D; ++d) acc[d] = 0.0f;
    // normal partners: candidate k of the flattened bin ranges (uniform trip count: the
    // shuffles below need every lane)
    for (int k0 = 0; k0 < total; k0 += 32) {
      const int k = k0 + lane;
      // owning bin: the first lane whose inclusive count exceeds k
      int o = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const int probe = o + step - 1;
        const int v = __shfl_sync(0xffffffffu, incl, probe < 31 ? probe : 31);
        if (probe < NB && v <= k) o += step;
      }
      const int base = __shfl_sync(0xffffffffu, incl - cnt, o);
      const int st = __shfl_sync(0xffffffffu, start, o);
      float of[D];
#pragma unroll
      for (int d = 0; d < D; ++d) of[d] = __shfl_sync(0xffffffffu, ofs[d], o);
      if (k >= total) continue;
      const int tt = static_cast<int>(a.perm[st + (k - base)] & 0xffffffffu);
      // the candidate's state, element id and record: independent loads, issued together
      const unsigned char stt = a.state[tt];
      const int ej = a.eid[tt];
      const float4 pj = a.pk[tt];
      if (stt != kSlotNormal || ej < 0 || (ej >> 1) == gf) continue;
      float dx[D];
      float r2 = 0.0f;
#pragma unroll
      for (int d = 0; d < D; ++d) {
        dx[d] = pk_c(pj, d) + of[d];
        r2 += dx[d] * dx[d];
      }
      const float f0 = pair_f0_fast<LAW>(r2, sf, fabsf(pj.w), eps, rcs, true, C.well_eps_f, C.well_sigma_f, C.force_shifted);
      if (f0 != 0.0f) {
#pragma unroll
        for (int d = 0; d < D; ++d) {
          acc[d] += f0 * dx[d];
          atomicAdd(&a.facc[d * SS + tt], -f0 * dx[d]);
        }
        atomicOr(&a.ftouch[tt >> 5], 1u << (tt & 31));
      }
    }
    // fresh partners: lane o walks the fresh list of bin o (current epoch only)
    if (bin >= 0) {
      unsigned long long ent = a.fhead[bin];
      for (int guard = 0; guard < kFreshCap && static_cast<unsigned>(ent >> 32) == epoch; ++guard) {
        const int q = static_cast<int>(ent & 0xffffffffu);
        ent = a.fnext[q];
        const unsigned char sq = a.state[q];
        const int eq = a.eid[q];
        const float4 pq = a.pk[q];
        if (q == f || sq != kSlotFresh || eq < 0 || (eq >> 1) == gf) continue;
        float dx[D];
        float r2 = 0.0f;
#pragma unroll
        for (int d = 0; d < D; ++d) {
          dx[d] = pk_c(pq, d) + ofs[d];
          r2 += dx[d] * dx[d];
        }
        const float f0 = pair_f0_fast<LAW>(r2, sf, fabsf(pq.w), eps, rcs, true, C.well_eps_f, C.well_sigma_f, C.force_shifted);
#pragma unroll
        for (int d = 0; d < D; ++d) acc[d] += f0 * dx[d];
      }
    }
#pragma unroll
    for (int d = 0; d < D; ++d) {
      float v = acc[d];
#pragma unroll
      for (int q = 16; q > 0; q >>= 1) v += __shfl_xor_sync(0xffffffffu, v, q);
      if (lane == 0) atomicAdd(&a.facc[d * SS + f], v);
    }
    if (lane == 0) atomicOr(&a.ftouch[f >> 5], 1u << (f & 31));
  }
}

template <int D>
void lists_d(const SkinArgs &a, int law, int grid, cudaStream_t s) {
  switch (law) {
    case CIL_FORCE_LJ_WCA:
      k_skin_lists<D, CIL_FORCE_LJ_WCA><<<grid, kTile, 0, s>>>(a);
      break;
    case CIL_FORCE_SOFTCORE:
      k_skin_lists<D, CIL_FORCE_SOFTCORE><<<grid, kTile, 0, s>>>(a);
      break;
    case CIL_FORCE_SC:
      k_skin_lists<D, CIL_FORCE_SC><<<grid, kTile, 0, s>>>(a);
      break;
    default:
      k_skin_lists<D, CIL_FORCE_HERTZ><<<grid, kTile, 0, s>>>(a);
      break;
  }
}

template <int D>
void fresh_d(const SkinArgs &a, int law, cudaStream_t s) {
  const int grid = a.grid;
  switch (law) {
    case CIL_FORCE_LJ_WCA:
      k_fresh_pairs<D, CIL_FORCE_LJ_WCA><<<grid, kFreshBlock, sizeof(int) * a.B, s>>>(a);
      break;
    case CIL_FORCE_SOFTCORE:
      k_fresh_pairs<D, CIL_FORCE_SOFTCORE><<<grid, kFreshBlock, sizeof(int) * a.B, s>>>(a);
      break;
    case CIL_FORCE_SC:
      k_fresh_pairs<D, CIL_FORCE_SC><<<grid, kFreshBlock, sizeof(int) * a.B, s>>>(a);
      break;
    default:
      k_fresh_pairs<D, CIL_FORCE_HERTZ><<<grid, kFreshBlock, sizeof(int) * a.B, s>>>(a);
      break;
  }
}

}  // namespace

void launch_skin_begin(const SkinArgs &a, cudaStream_t s) {
  k_skin_begin<<<(32 * a.B + 127) / 128, 128, 0, s>>>(a);
}

void launch_skin_rebin(const SkinArgs &a, int dim, int grid, cudaStream_t s) {
  if (dim == 2)
    k_skin_rebin<2><<<grid, kTile, 0, s>>>(a);
  else
    k_skin_rebin<3><<<grid, kTile, 0, s>>>(a);
}

void launch_list_flatten(const SkinArgs &a, int grid, cudaStream_t s) { k_list_flatten<<<grid, 128, 0, s>>>(a); }

void launch_skin_lists(const SkinArgs &a, int dim, int law, int grid, cudaStream_t s) {
  if (dim == 2)
    lists_d<2>(a, law, grid, s);
  else
    lists_d<3>(a, law, grid, s);
}

void launch_fresh_pairs(const SkinArgs &a, int dim, int law, cudaStream_t s) {
  if (dim == 2)
    fresh_d<2>(a, law, s);
  else
    fresh_d<3>(a, law, s);
}

}  // namespace cil
