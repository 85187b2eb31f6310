// Fused force + integrate kernels: one thread per binned element.
//
// Per element, in the reference's accumulation order (calculForcesPressure,
// CIL.cu:999-1007):
//   intra-cell spring + motility (binaryCellForce's role, MD.cu:525-598; assigns),
//   one-sided flat Hertz walls (Wall.hpp:80-91's role), passive noise zeta_j W
//   (CIL.cu:84-98), then pair forces from every other cell's elements in the 3^d
//   neighbour bins (calculInterForces + cellCellForce, CIL.cu:177-231, MD.cu:757-790,
//   as a full stencil: each thread accumulates only its own force, so no atomics), and
//   finally the overdamped Euler-Maruyama update with the reference's periodic wrap
//   (updatePositions, CIL.cu:858-875; BoundingBox::updatePos, Utils.hpp:561-566).
//
// FP64 form (k_force_fp64): everything in FP64; the parity path.
// Mixed form (k_force_mixed): GB300 issues FP64 at about 1/64 of the FP32 rate, so every
//   per-element operation runs in FP32 on bin-local coordinates (the element's FP32 offset
//   from its bin origin plus the FP32 offset between bin origins, exact for a periodic
//   image) and only the position accumulation stays FP64: one FP64 add per axis, with the
//   float->double conversion and the wrap test done in integer arithmetic.
#include "cil_internal.cuh"

namespace cil {

namespace {

template <int D>
__device__ __forceinline__ bool neighbor_bin(const ColonyConst &C, const int *bi, const int *o,
                                             int *nb, double *shift) {
#pragma unroll
  for (int d = 0; d < D; ++d) {
    int v = bi[d] + o[d];
    shift[d] = 0.0;
    if (v < 0) {
      if (!C.periodic[d]) return false;
      v += C.ns[d];
      shift[d] = -C.box[d];
    } else if (v >= C.ns[d]) {
      if (!C.periodic[d]) return false;
      v -= C.ns[d];
      shift[d] = C.box[d];
    }
    nb[d] = v;
  }
  return true;
}

template <int D>
__device__ __forceinline__ bool neighbor_bin_i(const ColonyConst &C, const int *bi, const int *o, int *nb) {
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

template <int D, int LAW>
__global__ void __launch_bounds__(kTile) k_force_fp64(ForceArgs a_) {
  ForceArgs a = a_;
  a.ts = *a_.ts_dev;
  const int total = a.tiles_live[a.B];
  for (int t = blockIdx.x; t < total; t += gridDim.x) {
    const int c = colony_of_tile(a.tiles_live, a.B, t);
    const ColonyConst &C = a.col[c];
    const int s = C.slot_base + (t - a.tiles_live[c]) * kTile + threadIdx.x;
    const int nlive = a.cnt[c].nlive;
    if (s >= C.slot_base + nlive) continue;

    const size_t SS = a.SS;
    const int e = a.eid[s];
    if (e < 0) continue;
    const int g = e >> 1, j = e & 1;
    double xi[D];
#pragma unroll
    for (int d = 0; d < D; ++d) xi[d] = a.x_in[d * SS + s];
    const double si = a.sig[s];

    double F[D];
    // ---- intra-cell: linear spring to the partner + motility along back->front
    {
      const int ps = a.slot_of[e ^ 1];
      double rij[D];
      double r2 = 0.0;
#pragma unroll
      for (int d = 0; d < D; ++d) {
        const double xp = a.x_in[d * SS + ps];
        double v = (j == 0) ? xp - xi[d] : xi[d] - xp;  // r1 - r0
        if (C.periodic[d]) v -= static_cast<double>(nint(v / C.box[d])) * C.box[d];
        rij[d] = v;
        r2 += v * v;
      }
      if (r2 == 0.0) {
#pragma unroll
        for (int d = 0; d < D; ++d) F[d] = 0.0;
      } else if (C.cell_sm && a.cst[g] == kCellDividing) {
        double spring, act[2];
        fene_bond_dividing<double>(r2, fmax(si, a.sig[ps]), C.fene_r2max_div, C.fene_kappa, C.fene_kappa_push,
                                   C.fene_ratio, C.div_r2min, C.growth_k0, C.growth_k1, C.growth_k2, spring, act);
        double rnd[3] = {0.0, 0.0, 0.0};
        if (C.act_noise && a.noise_mode == 2) bond_noise<D, double>(a.noise_act[g], a.noise_act_t[g], rij, sqrt(r2), rnd);
#pragma unroll
        for (int d = 0; d < D; ++d)
          F[d] = (j == 0) ? -(act[0] * rij[d] + spring * rij[d] * 1.0 + rnd[d] * rij[d])
                          : act[1] * rij[d] + spring * rij[d] * 1.0 + rnd[d] * rij[d];
      } else if (C.intra_fene) {
        const double r = sqrt(r2);
        double spring, sc;
        fene_bond<double>(r2, r, fmax(si, a.sig[ps]), C.fene_r2max, C.fene_kappa, C.fene_kappa_push, C.fene_ratio,
                          C.fene_rss, C.cil, spring, sc);
        double rnd[3] = {0.0, 0.0, 0.0};
        if (C.act_noise && a.noise_mode == 2) bond_noise<D, double>(a.noise_act[g], a.noise_act_t[g], rij, r, rnd);
#pragma unroll
        for (int d = 0; d < D; ++d) {
          const double nd = C.cil ? rij[d] : rij[d] * sc;
          F[d] = (j == 0) ? -(C.motility[0] * nd + spring * rij[d] * 2.0 + rnd[d] * rij[d])
                          : C.motility[1] * nd + spring * rij[d] * 2.0 + rnd[d] * rij[d];
        }
      } else {
        const double r = sqrt(r2);
        double rest = C.rest0;
        if (C.divide) {
          const int2 cy = a.cyc[s];
          const int span = cy.y - cy.x;
          double frac = span > 0 ? static_cast<double>(a.ts - cy.x) / static_cast<double>(span) : 1.0;
          frac = fmin(1.0, fmax(0.0, frac));
          rest = C.rest0 + (C.rest1 - C.rest0) * frac;
        }
        const double sp = C.kappa * (r - rest);
#pragma unroll
        for (int d = 0; d < D; ++d) {
          const double nd = rij[d] / r;
          F[d] = (j == 0) ? sp * nd - C.motility[0] * nd : -sp * nd + C.motility[1] * nd;
        }
      }
    }
    // ---- walls
    if (C.nwalls > 0) {
      const double rad = 0.5 * si;
      for (int w = 0; w < C.nwalls; ++w) {
        const double dir = static_cast<double>(C.wall_dir[w]);
        const double delta = rad - dir * (xi[D - 1] - C.wall_pos[w]);
        if (delta > 0.0) F[D - 1] += dir * C.wall_E * delta * sqrt(delta);
      }
    }
    // ---- passive noise
    if (a.noise_mode == 2) {
      const size_t base = static_cast<size_t>(C.noise_per_cell ? g : e) * D;
#pragma unroll
      for (int d = 0; d < D; ++d) F[d] += C.zeta[j] * a.noise[base + d];
    } else if (a.noise_mode == 1) {
      uint32_t w[4];
      noise_words<D>(e - 2 * C.cell_base, C.noise_per_cell, noise_index(a.ts, a.heun), C.rng_stream, a.seed_lo, a.seed_hi, w);
      float n[4];
      box_muller(w[0], w[1], n[0], n[1]);
      if (D == 3) box_muller(w[2], w[3], n[2], n[3]);
#pragma unroll
      for (int d = 0; d < D; ++d) F[d] += C.zeta[j] * (C.noise_amp * static_cast<double>(n[d]));
    }

    // ---- pair forces
    const double eps = C.epsilon, rcs = C.rcut_scale;
    if (C.single_bin) {
      // one bin: all elements, minimum image as BoundingBox::distance (Utils.hpp:536-544)
      for (int tt = C.slot_base; tt < C.slot_base + nlive; ++tt) {
        const int ej = a.eid[tt];
        if (ej < 0 || (ej >> 1) == g) continue;
        double dx[D];
        double r2 = 0.0;
#pragma unroll
        for (int d = 0; d < D; ++d) {
          double v = a.x_in[d * SS + tt] - xi[d];
          if (C.periodic[d]) v -= static_cast<double>(nint(v / C.box[d])) * C.box[d];
          dx[d] = v;
          r2 += v * v;
        }
        double f0;
        if (pair_force<LAW, double>(r2, si, a.sig[tt], eps, rcs, f0, C.well_eps, C.well_sigma, C.force_shifted)) {
#pragma unroll
          for (int d = 0; d < D; ++d) F[d] += f0 * dx[d];
        }
      }
    } else {
      int bi[D];
      bin_decode<D>(C, a.sbin[s], bi);
      // the partners inside the cutoff, in walk order with their neighbour bin: their pair
      // forces are evaluated kNear at a time after the walk, so the warp runs the FP64 law with
      // its lanes converged instead of once per candidate (the sums keep the walk order)
      const float sif = static_cast<float>(si), rcsf = static_cast<float>(rcs);
      const float xif = static_cast<float>(C.well_sigma);
      constexpr int kNear = 16;
      int near_t[kNear];
      unsigned char near_o[kNear];
      int nnear = 0;
      auto pairs = [&]() {
        for (int k = 0; k < nnear; ++k) {
          const int tt = near_t[k], code = near_o[k];
          const int oo[3] = {code % 3 - 1, (code / 3) % 3 - 1, code / 9 - 1};
          int nb[D];
          double shift[D];
          neighbor_bin<D>(C, bi, oo, nb, shift);
          double dx[D];
          double r2 = 0.0;
#pragma unroll
          for (int d = 0; d < D; ++d) {
            dx[d] = (__ldg(a.x_in + d * SS + tt) + shift[d]) - xi[d];
            r2 += dx[d] * dx[d];
          }
          double f0;
          if (pair_force<LAW, double>(r2, si, __ldg(a.sig + tt), eps, rcs, f0, C.well_eps, C.well_sigma,
                                      C.force_shifted)) {
#pragma unroll
            for (int d = 0; d < D; ++d) F[d] += f0 * dx[d];
          }
        }
        nnear = 0;
      };
      int o[3] = {-1, -1, -1};
      for (o[0] = -1; o[0] <= 1; ++o[0])
        for (o[1] = -1; o[1] <= 1; ++o[1])
          for (o[2] = (D == 3 ? -1 : 0); o[2] <= (D == 3 ? 1 : 0); ++o[2]) {
            int nb[D];
            double shift[D];
            if (!neighbor_bin<D>(C, bi, o, nb, shift)) continue;
            const int2 r = a.range[C.bin_base + bin_id<D>(C, nb)];
            const unsigned char code = static_cast<unsigned char>((o[0] + 1) + 3 * (o[1] + 1) + 9 * (o[2] + 1));
            for (int tt = r.x; tt < r.y; ++tt) {
              const int ej = __ldg(a.eid + tt);
              if (ej < 0 || (ej >> 1) == g) continue;
              // a conservative FP32 range test on the FP64 separation (pair_force repeats the
              // exact test): one FP64 subtraction per axis per candidate, the rest in FP32
              float r2f = 0.0f;
#pragma unroll
              for (int d = 0; d < D; ++d) {
                const float dx = static_cast<float>((__ldg(a.x_in + d * SS + tt) + shift[d]) - xi[d]);
                r2f += dx * dx;
              }
              if (!pair_maybe_in_range<LAW>(r2f, sif, static_cast<float>(__ldg(a.sig + tt)), rcsf, xif)) continue;
              near_t[nnear] = tt;
              near_o[nnear] = code;
              if (++nnear == kNear) pairs();
            }
          }
      pairs();
    }

    // ---- checks, integration, outputs
    bool finite = true;
#pragma unroll
    for (int d = 0; d < D; ++d) finite = finite && isfinite(F[d]);
    if (!finite) atomicOr(&a.cnt[c].err, kErrNan);
    if (a.frc) {
#pragma unroll
      for (int d = 0; d < D; ++d) a.frc[d * SS + s] = F[d];
    }
    if (a.integrate) {
      const double temp = a.heun ? 0.5 * C.temp[j] : C.temp[j];  // (dt/2) / zeta is exact
      bool inside = true;
#pragma unroll
      for (int d = 0; d < D; ++d) {
        const double tnew = __dadd_rn(xi[d], __dmul_rn(temp, F[d]));
        double xn;
        if (C.periodic[d]) {
          xn = wrap_like_fmod(tnew, C.box[d]);
        } else {
          xn = tnew;
          inside = inside && (xn >= 0.0 && xn < C.box[d]);
        }
        a.x_out[d * SS + s] = xn;
      }
      if (!inside) atomicOr(&a.cnt[c].err, kErrBox);
      if (a.vel) {
#pragma unroll
        for (int d = 0; d < D; ++d) {
          const double v = F[d] * C.mu_eff[j];
          a.vel[d * SS + s] = a.heun == 2 ? 0.5 * ((a.vel_prev ? a.vel_prev : a.vel)[d * SS + s] + v) : v;
        }
      }
    }
  }
}

// ---------------------------------------------------------------- mixed-precision pieces

// Intra-cell spring + motility, walls and passive noise of one element (FP32), in the
// reference's order. ui / bi: the element's packed coordinates and home bin.
template <int D>
__device__ __forceinline__ void mixed_own_forces(const ForceArgs &a, const ColonyConst &C, int s, int e,
                                                 const float *ui, const int *bi, float si, float *F) {
  const int g = e >> 1, j = e & 1;
  {
    const int ps = a.slot_of[e ^ 1];
    const float4 pp = a.pk[ps];
    int bp[D];
    bin_decode<D>(C, a.sbin[ps], bp);
    float rij[D];
    float r2 = 0.0f;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      float v = pk_c(pp, d) - ui[d];
      if (C.single_bin) {
        if (C.periodic[d]) v -= rintf(v * C.inv_bwf[d]) * C.bwf[d];
      } else {
        int db = bp[d] - bi[d];
        if (C.periodic[d]) {
          if (db > (C.ns[d] >> 1)) db -= C.ns[d];
          if (db < -(C.ns[d] >> 1)) db += C.ns[d];
        }
        v += static_cast<float>(db) * C.bwf[d];
      }
      rij[d] = (j == 0) ? v : -v;  // r1 - r0
      r2 += rij[d] * rij[d];
    }
#pragma unroll
    for (int d = 0; d < D; ++d) F[d] = 0.0f;
    if (r2 > 0.0f && C.cell_sm && a.cst[g] == kCellDividing) {
      float spring, act[2];
      fene_bond_dividing<float>(r2, fmaxf(si, fabsf(pp.w)), C.fene_r2max_div_f, C.fene_kappa_f, C.fene_kappa_push_f,
                                C.fene_ratio_f, C.div_r2min_f, C.growth_k0_f, C.growth_k1_f, C.growth_k2_f, spring, act);
      const float coef = (j == 0) ? -(act[0] + spring) : act[1] + spring;
      float rnd[3] = {0.0f, 0.0f, 0.0f};
      if (C.act_noise && a.noise_mode == 2)
        bond_noise<D, float>(static_cast<float>(a.noise_act[g]), static_cast<float>(a.noise_act_t[g]), rij, sqrtf(r2), rnd);
#pragma unroll
      for (int d = 0; d < D; ++d) F[d] = coef * rij[d] + (j == 0 ? -rnd[d] : rnd[d]) * rij[d];
    } else if (r2 > 0.0f && C.intra_fene) {
      const float rinv = rsqrtf(r2);
      float spring, sc;
      fene_bond<float>(r2, r2 * rinv, fmaxf(si, fabsf(pp.w)), C.fene_r2max_f, C.fene_kappa_f, C.fene_kappa_push_f,
                       C.fene_ratio_f, C.fene_rss_f, C.cil, spring, sc);
      const float coef = (j == 0) ? -(C.motility_f[0] * sc + 2.0f * spring) : C.motility_f[1] * sc + 2.0f * spring;
      float rnd[3] = {0.0f, 0.0f, 0.0f};
      if (C.act_noise && a.noise_mode == 2)
        bond_noise<D, float>(static_cast<float>(a.noise_act[g]), static_cast<float>(a.noise_act_t[g]), rij, r2 * rinv, rnd);
#pragma unroll
      for (int d = 0; d < D; ++d) F[d] = coef * rij[d] + (j == 0 ? -rnd[d] : rnd[d]) * rij[d];
    } else if (r2 > 0.0f) {
      const float rinv = rsqrtf(r2);
      float rest = C.rest0_f;
      if (C.divide) {
        const int2 cy = a.cyc[s];
        const int span = cy.y - cy.x;
        float frac = span > 0 ? __fdividef(static_cast<float>(a.ts - cy.x), static_cast<float>(span)) : 1.0f;
        frac = fminf(1.0f, fmaxf(0.0f, frac));
        rest = C.rest0_f + (C.rest1_f - C.rest0_f) * frac;
      }
      const float sp = C.kappa_f * (r2 * rinv - rest);
      const float coef = ((j == 0) ? (sp - C.motility_f[0]) : (C.motility_f[1] - sp)) * rinv;
#pragma unroll
      for (int d = 0; d < D; ++d) F[d] = coef * rij[d];
    }
  }
  if (C.nwalls > 0) {
    const float z = static_cast<float>(bi[D - 1]) * C.bwf[D - 1] + ui[D - 1];
    const float rad = 0.5f * si;
    for (int w = 0; w < C.nwalls; ++w) {
      const float dir = static_cast<float>(C.wall_dir[w]);
      const float delta = rad - dir * (z - C.wall_pos_f[w]);
      if (delta > 0.0f) F[D - 1] += dir * C.wall_E_f * delta * (delta * rsqrtf(delta));
    }
  }
  if (a.noise_mode == 1) {
    // Box-Muller with the fast log / sincos
    uint32_t w[4];
    noise_words<D>(e - 2 * C.cell_base, C.noise_per_cell, noise_index(a.ts, a.heun), C.rng_stream, a.seed_lo, a.seed_hi, w);
    const float amp = C.zeta_f[j] * C.amp_f;
#pragma unroll
    for (int h = 0; h < (D + 1) / 2; ++h) {
      const float u1 = static_cast<float>((w[2 * h] >> 8) + 1u) * 5.9604644775390625e-08f;
      const float u2 = static_cast<float>(w[2 * h + 1] >> 8) * 5.9604644775390625e-08f;
      const float m = fmaxf(-2.0f * __logf(u1), 0.0f);
      const float rad = m * rsqrtf(fmaxf(m, 1e-30f));  // sqrt(m), 0 when u1 == 1
      float sn, cs;
      __sincosf(6.2831853071795865f * u2, &sn, &cs);
      F[2 * h] += amp * rad * cs;
      if (2 * h + 1 < D) F[2 * h + 1] += amp * rad * sn;
    }
  } else if (a.noise_mode == 2) {
    const size_t base = static_cast<size_t>(C.noise_per_cell ? g : e) * D;
#pragma unroll
    for (int d = 0; d < D; ++d) F[d] += C.zeta_f[j] * static_cast<float>(a.noise[base + d]);
  }
}

// Checks, outputs and the Euler-Maruyama update of one element: one FP64 add per axis, the
// float->double conversion and the periodic wrap in integer arithmetic. Writes the next
// packed record (w carried over) and returns the FP32 step in dx.
template <int D>
__device__ __forceinline__ void mixed_integrate(const ForceArgs &a, const ColonyConst &C, int c, int s, int j,
                                                const float *ui, float w, const float *F, float *dx) {
  bool finite = true;
#pragma unroll
  for (int d = 0; d < D; ++d) finite = finite && isfinite(F[d]);
  if (!finite) atomicOr(&a.cnt[c].err, kErrNan);
  if (a.frc) {
#pragma unroll
    for (int d = 0; d < D; ++d) a.frc[d * a.SS + s] = static_cast<double>(F[d]);
  }
  if (!a.integrate) return;
  const float temp = a.heun ? 0.5f * C.temp_f[j] : C.temp_f[j];
  bool inside = true;
  float4 pn = make_float4(0.0f, 0.0f, 0.0f, w);
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const float dxf = temp * F[d];
    double xn = a.x_in[d * a.SS + s] + f2d_exact(dxf);
    const long long xb = __double_as_longlong(xn);
    const long long lb = __double_as_longlong(C.box[d]);
    const bool lo = xb < 0, hi = xb >= lb;
    if (C.periodic[d]) {
      // non-negative doubles order like their bit patterns: wrap tests without FP64
      // compares; a tiny negative x + L that rounds to L ends at 0 like fmod(x + L, L). The
      // wrap runs only in warps where some element crossed 0 or L.
      if (__any_sync(__activemask(), lo || hi)) {
        if (lo) xn = (xb & 0x7fffffffffffffffll) ? xn + C.box[d] : 0.0;
        if (__double_as_longlong(xn) >= lb) xn -= C.box[d];
      }
    } else {
      inside = inside && !lo && !hi;
    }
    a.x_out[d * a.SS + s] = xn;
    pk_set(pn, d, ui[d] + dxf);
    dx[d] = dxf;
  }
  a.pk_next[s] = pn;
  if (!inside) atomicOr(&a.cnt[c].err, kErrBox);
  if (a.vel) {
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const double v = static_cast<double>(F[d] * C.mu_f[j]);
      a.vel[d * a.SS + s] = a.heun == 2 ? 0.5 * ((a.vel_prev ? a.vel_prev : a.vel)[d * a.SS + s] + v) : v;
    }
  }
}

// Mixed-precision step without lists, one CTA per tile of kTile consecutive binned elements:
//  1. each thread: its element's intra-cell, wall and noise force (FP32) and the ranges of
//     its 3^d neighbour bins, staged in shared memory with the candidate count;
//  2. a block scan turns the counts into one list of (element, candidate) pairs and every
//     thread evaluates an equal contiguous chunk of it, so lanes stay converged whatever
//     the bin occupancies; partial sums are added into the element's shared accumulator;
//  3. each thread adds its element's pair force and integrates.
template <int D, int LAW>
__global__ void __launch_bounds__(kTile) k_force_mixed(ForceArgs a_) {
  ForceArgs a = a_;
  a.ts = *a_.ts_dev;
  constexpr int NB = (D == 2) ? 9 : 27;
  extern __shared__ int smem[];
  int *s_start = smem;                       // [NB][kTile]
  int *s_cnt = s_start + NB * kTile;         // [NB][kTile]
  int *s_off = s_cnt + NB * kTile;           // [kTile + 1]
  int *s_g = s_off + kTile + 1;              // [kTile]
  float *s_u = reinterpret_cast<float *>(s_g + kTile);  // [D][kTile]
  float *s_si = s_u + D * kTile;             // [kTile]
  float *s_F = s_si + kTile;                 // [D][kTile]
  __shared__ int s_total;

  const int tid = threadIdx.x;
  const int total = a.tiles_live[a.B];
  for (int t = blockIdx.x; t < total; t += gridDim.x) {
    const int c = colony_of_tile(a.tiles_live, a.B, t);
    const ColonyConst &C = a.col[c];
    const int s = C.slot_base + (t - a.tiles_live[c]) * kTile + tid;
    const int nlive = a.cnt[c].nlive;
    const int e = s < C.slot_base + nlive ? a.eid[s] : -1;
    const bool live = e >= 0;
    const int g = live ? (e >> 1) : -1;
    const int j = e & 1;

    float ui[D], F[D];
    float si = 0.0f, w = 0.0f;
    int bi[D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      ui[d] = 0.0f;
      F[d] = 0.0f;
      bi[d] = 0;
    }
    int ncand = 0;
    if (live) {
      const float4 pi = a.pk[s];
#pragma unroll
      for (int d = 0; d < D; ++d) ui[d] = pk_c(pi, d);
      w = pi.w;
      si = fabsf(w);
      bin_decode<D>(C, a.sbin[s], bi);
      mixed_own_forces<D>(a, C, s, e, ui, bi, si, F);
      // ---- neighbour bin ranges
      if (!C.single_bin) {
#pragma unroll
        for (int o = 0; o < NB; ++o) {
          int off[3] = {o / (D == 2 ? 3 : 9) - 1, (D == 2 ? o % 3 : (o / 3) % 3) - 1, (D == 2 ? 0 : o % 3 - 1)};
          int nb[D];
          int st = 0, n = 0;
          if (neighbor_bin_i<D>(C, bi, off, nb)) {
            const int2 r = a.range[C.bin_base + bin_id<D>(C, nb)];
            st = r.x;
            n = r.y - r.x;
          }
          s_start[o * kTile + tid] = st;
          s_cnt[o * kTile + tid] = n;
          ncand += n;
        }
      }
    }
    if (!live || C.single_bin) {
#pragma unroll
      for (int o = 0; o < NB; ++o) s_cnt[o * kTile + tid] = 0;
    }
#pragma unroll
    for (int d = 0; d < D; ++d) {
      s_u[d * kTile + tid] = ui[d];
      s_F[d * kTile + tid] = 0.0f;
    }
    s_si[tid] = si;
    s_g[tid] = g;
    // ---- pair list offsets
    {
      const int lane = tid & 31, wid = tid >> 5;
      int inc = ncand;
#pragma unroll
      for (int q = 1; q < 32; q <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, inc, q);
        if (lane >= q) inc += v;
      }
      __shared__ int ws[kTile / 32];
      if (lane == 31) ws[wid] = inc;
      __syncthreads();
      if (wid == 0) {
        int wv = lane < kTile / 32 ? ws[lane] : 0;
#pragma unroll
        for (int q = 1; q < 32; q <<= 1) {
          const int v = __shfl_up_sync(0xffffffffu, wv, q);
          if (lane >= q) wv += v;
        }
        if (lane < kTile / 32) ws[lane] = wv;
        if (lane == kTile / 32 - 1) s_total = wv;
      }
      __syncthreads();
      s_off[tid] = (wid > 0 ? ws[wid - 1] : 0) + inc - ncand;
      __syncthreads();
    }
    // ---- pair chunk of this thread
    const int npairs = s_total;
    const float eps = C.eps_f, rcs = C.rcs_f;
    if (npairs > 0) {
      const int q = (npairs + kTile - 1) / kTile;
      int p = tid * q;
      const int p1 = min(p + q, npairs);
      if (p < p1) {
        // home element: largest i with s_off[i] <= p
        int lo = 0, hi = kTile - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (s_off[mid] <= p)
            lo = mid;
          else
            hi = mid - 1;
        }
        int i = lo;
        int k = p - s_off[i];
        int o = 0;
        while (k >= s_cnt[o * kTile + i]) {
          k -= s_cnt[o * kTile + i];
          ++o;
        }
        int tt = s_start[o * kTile + i] + k;
        int rem = s_cnt[o * kTile + i] - k;
        float uh[D], offv[D], acc[D];
        float sh = s_si[i];
        int gh = s_g[i];
#pragma unroll
        for (int d = 0; d < D; ++d) {
          uh[d] = s_u[d * kTile + i];
          acc[d] = 0.0f;
        }
        auto set_off = [&](int oo) {
          const int o0 = oo / (D == 2 ? 3 : 9) - 1;
          const int o1 = (D == 2 ? oo % 3 : (oo / 3) % 3) - 1;
          offv[0] = static_cast<float>(o0) * C.bwf[0] - uh[0];
          offv[1] = static_cast<float>(o1) * C.bwf[1] - uh[1];
          if (D == 3) offv[D - 1] = static_cast<float>(oo % 3 - 1) * C.bwf[D - 1] - uh[D - 1];
        };
        set_off(o);
        for (;;) {
          const int ej = __ldg(a.eid + tt);
          const float4 pj = __ldg(a.pk + tt);
          float dx[D];
          float r2 = 0.0f;
#pragma unroll
          for (int d = 0; d < D; ++d) {
            dx[d] = pk_c(pj, d) + offv[d];
            r2 += dx[d] * dx[d];
          }
          const float f0 = pair_f0_fast<LAW>(r2, sh, pj.w, eps, rcs, ej >= 0 && (ej >> 1) != gh, C.well_eps_f, C.well_sigma_f, C.force_shifted);
#pragma unroll
          for (int d = 0; d < D; ++d) acc[d] += f0 * dx[d];
          if (++p >= p1) break;
          ++tt;
          --rem;
          while (rem == 0) {
            if (++o == NB) {
#pragma unroll
              for (int d = 0; d < D; ++d) {
                atomicAdd(&s_F[d * kTile + i], acc[d]);
                acc[d] = 0.0f;
              }
              ++i;
              o = 0;
              sh = s_si[i];
              gh = s_g[i];
#pragma unroll
              for (int d = 0; d < D; ++d) uh[d] = s_u[d * kTile + i];
            }
            rem = s_cnt[o * kTile + i];
            tt = s_start[o * kTile + i];
            if (rem) set_off(o);
          }
        }
#pragma unroll
        for (int d = 0; d < D; ++d) atomicAdd(&s_F[d * kTile + i], acc[d]);
      }
    }
    __syncthreads();

    if (live) {
      if (C.single_bin) {
        // one bin only (tiny boxes): every element, FP32 minimum image
        for (int tt = C.slot_base; tt < C.slot_base + nlive; ++tt) {
          const int ej = a.eid[tt];
          const float4 pj = a.pk[tt];
          float dx[D];
          float r2 = 0.0f;
#pragma unroll
          for (int d = 0; d < D; ++d) {
            float v = pk_c(pj, d) - ui[d];
            if (C.periodic[d]) v -= rintf(v * C.inv_bwf[d]) * C.bwf[d];
            dx[d] = v;
            r2 += v * v;
          }
          const float f0 = pair_f0_fast<LAW>(r2, si, pj.w, eps, rcs, ej >= 0 && (ej >> 1) != g, C.well_eps_f, C.well_sigma_f, C.force_shifted);
#pragma unroll
          for (int d = 0; d < D; ++d) F[d] += f0 * dx[d];
        }
      } else {
#pragma unroll
        for (int d = 0; d < D; ++d) F[d] += s_F[d * kTile + tid];
      }
      float dstep[D];
      mixed_integrate<D>(a, C, c, s, j, ui, w, F, dstep);
    }
    __syncthreads();
  }
}

// Asynchronous global -> shared copies (cp.async, sm_80 and later): issued early, waited for
// where the data is used, so their latency overlaps the work in between. Each thread waits
// for its own copies; a __syncwarp after the wait publishes them to the warp.
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Per-warp shared memory of the cell kernel, for segments of SEG flattened list entries:
//   records of the warp's 64 elements             64 x 16 B
//   FP64 positions of the 64 elements (staged)    64 x D x 8 B, axis-major
//   list entries of the segment                   SEG x 4 B
//   owner (element of the warp) of each entry     SEG x 1 B
//   pair force of each entry                      SEG x D x 4 B
// SEG is the largest multiple of 32 (at most 1024) with which MINB blocks of TILE threads fit
// in the 228 KB of shared memory of an SM, leaving 2 KB per block for the static variables
// and the per-block reservation.
template <int D, int MINB, int TILE>
__host__ __device__ constexpr int pair_seg() {
  return ((233472 / MINB - 2048) / (TILE / 32) - (64 * 16 + 64 * D * 8)) / (5 + 4 * D) / 32 * 32 > 1024
             ? 1024
             : ((233472 / MINB - 2048) / (TILE / 32) - (64 * 16 + 64 * D * 8)) / (5 + 4 * D) / 32 * 32;
}
template <int D, int SEG>
__host__ __device__ constexpr int pair_smem_warp() {
  return 64 * 16 + 64 * D * 8 + SEG * (4 + 1 + 4 * D);
}
template <int D, int SEG>
struct PairSmem {
  float4 *rec;
  double *x;
  unsigned *ent;
  unsigned char *own;
  float *c;
  __device__ __forceinline__ explicit PairSmem(unsigned char *w)
      : rec(reinterpret_cast<float4 *>(w)),
        x(reinterpret_cast<double *>(w + 64 * 16)),
        ent(reinterpret_cast<unsigned *>(w + 64 * 16 + 64 * D * 8)),
        own(w + 64 * 16 + 64 * D * 8 + SEG * 4),
        c(reinterpret_cast<float *>(w + 64 * 16 + 64 * D * 8 + SEG * 5)) {}
};

// Bin-origin offsets by list-entry code (2 bits per axis: bin offset + 1), per block:
// entry k holds ((k >> 2d) & 3) - 1 times the bin width on axis d (exact products).
template <int D>
constexpr int kOffStride = D == 2 ? 2 : 4;
template <int D>
constexpr int kOffCodes = D == 2 ? 16 : 64;

// The warp's range of flattened list entries (k_list_flatten): element 2 lane owns [st0, en0),
// element 2 lane + 1 owns [st1, en1) of the warp's T entries. T and the starts are those of the
// last list build; an element that became fresh or dead since has an empty range (its entries
// are still evaluated, and dropped).
struct PairRange {
  int st0, en0, st1, en1, T;
};

// One segment [S, E) of the warp's range: 16-byte copies of its list entries and their owners
// from the flattened lists. The warp's range starts 16 KB aligned and S is a multiple of 32, so
// every copy is aligned; the copies round E up to 4 entries and 16 owners, which stays inside
// the warp's 64 kListCap entries and inside the segment's shared arrays (SEG is a multiple of 32).
template <int D, int SEG>
__device__ __forceinline__ void pairs_segment_start(const ForceArgs &a, int sw0, const PairRange &R, int S,
                                                    const PairSmem<D, SEG> &sm) {
  const int lane = threadIdx.x & 31;
  const int E = min(R.T, S + SEG);
  const int *le = a.lflat + static_cast<size_t>(sw0) * kListCap + S;
  const unsigned char *lo = a.oflat + static_cast<size_t>(sw0) * kListCap + S;
  const int ne = (E - S + 3) >> 2, no = (E - S + 15) >> 4;
  for (int i = lane; i < ne; i += 32) cp_async16(sm.ent + 4 * i, le + 4 * i);
  for (int i = lane; i < no; i += 32) cp_async16(sm.own + 16 * i, lo + 16 * i);
}

// The start of the pair pass, right after the cell's own loads: the records of the warp's 64
// elements into shared memory, the warp's range, and the copies of the first segment. Every
// lane calls it; lanes without a live cell pass n = (0, 0). ls: the two elements' starts;
// Tw: the warp's entry count at the last build.
template <int D, int SEG>
__device__ __forceinline__ PairRange pairs_begin(const ForceArgs &a, int sw0, int2 nn, ushort2 ls, int Tw,
                                                 const float4 *pr, const PairSmem<D, SEG> &sm) {
  const int lane = threadIdx.x & 31;
  sm.rec[2 * lane] = pr[0];
  sm.rec[2 * lane + 1] = pr[1];
  PairRange R;
  R.T = min(Tw, 64 * kListCap);
  R.st0 = ls.x;
  R.en0 = ls.x + nn.x;
  R.st1 = ls.y;
  R.en1 = ls.y + nn.y;
  pairs_segment_start<D, SEG>(a, sw0, R, 0, sm);
  return R;
}

// The pair forces of a warp's 32 cells (64 elements), whole warp: the elements' Verlet-list
// entries are taken as one flattened range (element by element, each list in order), so every
// lane evaluates a real entry whatever the lengths of the lists; each lane then adds its two
// elements' pair forces in list order (the sums do not depend on scheduling). UNROLL chunks of
// 32 entries have their partner records in flight together.
template <int D, int LAW, int UNROLL, int SEG>
__device__ __forceinline__ void pairs_finish(const ForceArgs &a, const ColonyConst &C, int sw0, const PairRange &R,
                                             float (*F)[D], const PairSmem<D, SEG> &sm, const float *s_off) {
  const int lane = threadIdx.x & 31;
  const float eps = C.eps_f, rcs = C.rcs_f;
  for (int S = 0; S < R.T; S += SEG) {  // uniform
    const int E = min(R.T, S + SEG);
    if (S > 0) {
      __syncwarp();  // the last segment's sums are read
      pairs_segment_start<D, SEG>(a, sw0, R, S, sm);
    }
    cp_async_wait_all();
    __syncwarp();  // every lane's copies (entries, records, owners) are visible to the warp
    for (int base = S; base < E; base += 32 * UNROLL) {  // uniform
      unsigned ent[UNROLL];
      int own[UNROLL];
      float4 pj[UNROLL];
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) {
        const int f = base + 32 * u + lane;
        own[u] = f < E ? sm.own[f - S] : -1;
        ent[u] = f < E ? sm.ent[f - S] : 0u;
      }
#pragma unroll
      for (int u = 0; u < UNROLL; ++u)
        pj[u] = own[u] >= 0 ? __ldg(a.pk + (ent[u] & ((1u << kListSlotBits) - 1u)))
                            : make_float4(0.0f, 0.0f, 0.0f, -1.0f);
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) {
        if (own[u] < 0) continue;
        const float4 me = sm.rec[own[u]];
        // the offset between the two home bins' origins, from the entry's bin offset code
        const float *ov = s_off + (ent[u] >> kListSlotBits) * kOffStride<D>;
        float dx[D];
        float r2 = 0.0f;
#pragma unroll
        for (int d = 0; d < D; ++d) {
          dx[d] = pk_c(pj[u], d) + (ov[d] - pk_c(me, d));
          r2 += dx[d] * dx[d];
        }
        const float f0 = pair_f0_fast<LAW>(r2, fabsf(me.w), pj[u].w, eps, rcs, pj[u].w > 0.0f, C.well_eps_f, C.well_sigma_f, C.force_shifted);
        float *cf = sm.c + (base + 32 * u + lane - S) * D;
#pragma unroll
        for (int d = 0; d < D; ++d) cf[d] = f0 * dx[d];
      }
    }
    __syncwarp();
    // each element adds its entries of the segment, in list order
    for (int f = max(R.st0, S); f < min(R.en0, E); ++f)
#pragma unroll
      for (int d = 0; d < D; ++d) F[0][d] += sm.c[(f - S) * D + d];
    for (int f = max(R.st1, S); f < min(R.en1, E); ++f)
#pragma unroll
      for (int d = 0; d < D; ++d) F[1][d] += sm.c[(f - S) * D + d];
  }
  cp_async_wait_all();  // a warp without list entries has waited for nothing yet
}

// Skin-mode step over cell-major slots, one thread per cell. Between slot re-sorts a cell's
// two elements sit in adjacent slots, back element first (s0 = slot_base + 2 p, s1 = s0 + 1):
// the re-sort ranks cells, division appends daughters as slot pairs, apoptosis leaves pairs of
// tombstones. So a thread reads both records, the cycle and the FP64 positions of its cell
// with coalesced loads, evaluates the intra-cell spring once and draws the noise of both
// elements from one Philox block (2D); the warp evaluates its 64 elements' Verlet-list
// entries as one flattened range (pairs_begin / pairs_finish). The list entries and the FP64
// positions are copied into shared memory asynchronously at the start, so they arrive while
// the spring, wall and noise terms are evaluated; in the pair pass only the partner records
// are gathered (UNROLL chunks of 32 entries in flight per warp). Per element: the spring, wall
// and noise terms are the expressions of the other force kernels, the pair terms are summed in
// list order, and pairs with fresh elements (created or moved by a division since the last
// list build, in no list) arrive through facc from k_fresh_pairs.
template <int D, int LAW, int UNROLL, int MINB, int TILE>
__global__ void __launch_bounds__(TILE, MINB) k_force_cells(const ForceArgs a) {
  constexpr int SEG = pair_seg<D, MINB, TILE>();
  extern __shared__ __align__(16) unsigned char s_pairs[];
  __shared__ ColonyConst sC;
  __shared__ unsigned s_dmax, s_smax;  // float bits of non-negative values
  __shared__ float s_ssum;
  __shared__ float s_half2;
  __shared__ int s_nbuilt;
  __shared__ int s_warps_done;
  __shared__ __align__(16) float s_off[kOffCodes<D> * kOffStride<D>];
  const int t = blockIdx.x;
  if (t >= a.tiles[a.B]) return;  // uniform per block (tiles over slot pairs)
  const int tid = threadIdx.x;
  const int c = colony_of_tile(a.tiles, a.B, t);
  {
    const int *src = reinterpret_cast<const int *>(a.col + c);
    int *dst = reinterpret_cast<int *>(&sC);
    for (int i = tid; i < static_cast<int>(sizeof(ColonyConst) / sizeof(int)); i += TILE) dst[i] = __ldg(src + i);
    if (tid < kOffCodes<D>) {
#pragma unroll
      for (int d = 0; d < D; ++d)
        s_off[tid * kOffStride<D> + d] = static_cast<float>(((tid >> (2 * d)) & 3) - 1) * __ldg(&a.col[c].bwf[d]);
    }
    if (tid == 0) {
      s_dmax = 0u;
      s_smax = 0u;
      s_ssum = 0.0f;
      s_half2 = a.skin[c].half2;
      s_nbuilt = a.skin[c].nslot_built;
      s_warps_done = 0;
    }
  }
  __syncthreads();
  const ColonyConst &C = sC;
  const int ts = __ldg(a.ts_dev);
  const size_t SS = a.SS;
  const int s0 = C.slot_base + 2 * ((t - a.tiles[c]) * TILE + tid);
  // every load of the cell is issued at once, guarded by the colony's slot capacity only (the
  // memory is there; what lies past the used slots is not used), so none waits on another
  const bool incap = s0 < C.slot_base + C.slot_cap;
  int2 ee = make_int2(-1, -1), sb = make_int2(0, 0), nn = make_int2(0, 0), cy = make_int2(0, 0);
  float4 pr[2] = {make_float4(0.0f, 0.0f, 0.0f, 0.0f), make_float4(0.0f, 0.0f, 0.0f, 0.0f)};
  ushort2 ls = make_ushort2(0, 0);
  if (incap) {
    ee = __ldg(reinterpret_cast<const int2 *>(a.eid + s0));
    pr[0] = __ldg(a.pk + s0);
    pr[1] = __ldg(a.pk + s0 + 1);
    sb = __ldg(reinterpret_cast<const int2 *>(a.sbin + s0));
    nn = __ldg(reinterpret_cast<const int2 *>(a.ncnt + s0));
    ls = __ldg(reinterpret_cast<const ushort2 *>(a.lstart + s0));
    if (C.divide) cy = __ldg(a.cyc + s0);
  }
  // the warp's entry count at the last build (warps past the slots of that build have none)
  const int sw0 = s0 - 2 * (tid & 31);
  const int Tw = sw0 < C.slot_base + s_nbuilt ? __ldg(a.lwarp + (sw0 >> 6)) : 0;
  // fresh-pair contributions: one bit per slot; slot bases are 32-aligned and s0 is even, so
  // both bits of the cell sit in one word (16 cells per word)
  const unsigned tword = a.ftouch[s0 >> 5];
  const unsigned tbits = (tword >> (s0 & 31)) & 3u;
  const bool used = s0 < C.slot_base + a.cnt[c].nslot;
  const bool live = used && ee.x >= 0;
  if (!live) nn = make_int2(0, 0);
  if (a.collect_due && C.divide) {  // uniform
    // cells whose cycle ends at the coming events (step ts + 1) join the colony's due-cell
    // queue: one atomic per warp
    const bool due = live && cy.y == ts + 1;
    const unsigned dm = __ballot_sync(0xffffffffu, due);
    if (dm) {
      const int lane = tid & 31, leader = __ffs(dm) - 1;
      int base = 0;
      if (lane == leader) base = atomicAdd(&a.cnt[c].ndue, __popc(dm));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (due) a.dueq[C.due_base + base + __popc(dm & ((1u << lane) - 1u))] = (ee.x >> 1) - C.cell_base;
    }
  }
  float d2 = 0.0f, st2[2] = {0.0f, 0.0f};
  // ---- the pair pass starts: the warp's records, its flattened list range, and asynchronous
  // copies of its list entries and of the cells' FP64 positions, which arrive while the
  // per-element terms below are evaluated
  PairSmem<D, SEG> sm(s_pairs + (tid >> 5) * pair_smem_warp<D, SEG>());
  const PairRange R = pairs_begin<D, SEG>(a, sw0, nn, ls, Tw, pr, sm);
  if (live) {
#pragma unroll
    for (int d = 0; d < D; ++d) cp_async16(sm.x + d * 64 + 2 * (tid & 31), a.x_in + d * SS + s0);
  }
  // ---- the per-element terms (live cells)
  float F[2][D], ui[2][D];
#pragma unroll
  for (int d = 0; d < D; ++d) F[0][d] = F[1][d] = 0.0f;
  if (live) {
    const int g = ee.x >> 1;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      ui[0][d] = pk_c(pr[0], d);
      ui[1][d] = pk_c(pr[1], d);
    }
    const float si[2] = {fabsf(pr[0].w), fabsf(pr[1].w)};
    int bi[2][D];
    bin_decode<D>(C, sb.x, bi[0]);
    bin_decode<D>(C, sb.y, bi[1]);
    // ---- intra-cell spring + motility (the back element's view r1 - r0; the front
    // element's is the same vector, as -(r0 - r1) is exact)
    {
      float rij[D];
      float r2 = 0.0f;
#pragma unroll
      for (int d = 0; d < D; ++d) {
        float v = ui[1][d] - ui[0][d];
        if (C.single_bin) {
          if (C.periodic[d]) v -= rintf(v * C.inv_bwf[d]) * C.bwf[d];
        } else {
          int db = bi[1][d] - bi[0][d];
          if (C.periodic[d]) {
            if (db > (C.ns[d] >> 1)) db -= C.ns[d];
            if (db < -(C.ns[d] >> 1)) db += C.ns[d];
          }
          v += static_cast<float>(db) * C.bwf[d];
        }
        rij[d] = v;
        r2 += v * v;
      }
      if (r2 > 0.0f && C.intra_fene) {
        const float rinv = rsqrtf(r2);
        float spring, sc;
        fene_bond<float>(r2, r2 * rinv, fmaxf(si[0], si[1]), C.fene_r2max_f, C.fene_kappa_f, C.fene_kappa_push_f,
                         C.fene_ratio_f, C.fene_rss_f, C.cil, spring, sc);
        const float coef0 = -(C.motility_f[0] * sc + 2.0f * spring);
        const float coef1 = C.motility_f[1] * sc + 2.0f * spring;
#pragma unroll
        for (int d = 0; d < D; ++d) {
          F[0][d] += coef0 * rij[d];
          F[1][d] += coef1 * rij[d];
        }
      } else if (r2 > 0.0f) {
        const float rinv = rsqrtf(r2);
        float rest = C.rest0_f;
        if (C.divide) {
          const int span = cy.y - cy.x;
          float frac = span > 0 ? __fdividef(static_cast<float>(ts - cy.x), static_cast<float>(span)) : 1.0f;
          frac = fminf(1.0f, fmaxf(0.0f, frac));
          rest = C.rest0_f + (C.rest1_f - C.rest0_f) * frac;
        }
        const float sp = C.kappa_f * (r2 * rinv - rest);
        const float coef0 = (sp - C.motility_f[0]) * rinv;
        const float coef1 = (C.motility_f[1] - sp) * rinv;
#pragma unroll
        for (int d = 0; d < D; ++d) {
          F[0][d] += coef0 * rij[d];
          F[1][d] += coef1 * rij[d];
        }
      }
    }
    // ---- walls
    if (C.nwalls > 0) {
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const float z = static_cast<float>(bi[j][D - 1]) * C.bwf[D - 1] + ui[j][D - 1];
        const float rad = 0.5f * si[j];
        for (int w = 0; w < C.nwalls; ++w) {
          const float dir = static_cast<float>(C.wall_dir[w]);
          const float delta = rad - dir * (z - C.wall_pos_f[w]);
          if (delta > 0.0f) F[j][D - 1] += dir * C.wall_E_f * delta * (delta * rsqrtf(delta));
        }
      }
    }
    // ---- passive noise
    if (a.noise_mode == 1) {
      uint32_t w[2][4];
      noise_words_cell<D>(g - C.cell_base, C.noise_per_cell, noise_index(ts, a.heun), C.rng_stream, a.seed_lo, a.seed_hi,
                              w[0], w[1]);
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const float amp = C.zeta_f[j] * C.amp_f;
#pragma unroll
        for (int h = 0; h < (D + 1) / 2; ++h) {
          const float u1 = static_cast<float>((w[j][2 * h] >> 8) + 1u) * 5.9604644775390625e-08f;
          const float u2 = static_cast<float>(w[j][2 * h + 1] >> 8) * 5.9604644775390625e-08f;
          const float m = fmaxf(-2.0f * __logf(u1), 0.0f);
          const float rad = m * rsqrtf(fmaxf(m, 1e-30f));  // sqrt(m), 0 when u1 == 1
          float sn, cs;
          __sincosf(6.2831853071795865f * u2, &sn, &cs);
          F[j][2 * h] += amp * rad * cs;
          if (2 * h + 1 < D) F[j][2 * h + 1] += amp * rad * sn;
        }
      }
    } else if (a.noise_mode == 2) {
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const size_t base = static_cast<size_t>(C.noise_per_cell ? g : 2 * g + j) * D;
#pragma unroll
        for (int d = 0; d < D; ++d) F[j][d] += C.zeta_f[j] * static_cast<float>(__ldg(a.noise + base + d));
      }
    }
  }
  // ---- pair forces from the Verlet lists: the whole warp
  pairs_finish<D, LAW, UNROLL, SEG>(a, C, sw0, R, F, sm, s_off);
  if (live) {
    double xin[2][D];
    float uref[2][D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      // this lane's own staged copies (complete: pairs_finish waited for them)
      const double2 xv = *reinterpret_cast<const double2 *>(sm.x + d * 64 + 2 * (tid & 31));
      xin[0][d] = xv.x;
      xin[1][d] = xv.y;
      if (tbits & 1u) F[0][d] += a.facc[d * SS + s0];
      if (tbits & 2u) F[1][d] += a.facc[d * SS + s0 + 1];
    }
    if (D == 2) {
      uref_unpack2(C.uq_inv, pr[0].z, uref[0]);
      uref_unpack2(C.uq_inv, pr[1].z, uref[1]);
    } else {
#pragma unroll
      for (int d = 0; d < D; ++d) {
        const float2 uv = __ldg(reinterpret_cast<const float2 *>(a.uref + d * SS + s0));
        uref[0][d] = uv.x;
        uref[1][d] = uv.y;
      }
    }
    // ---- checks, update (one FP64 add per axis, integer wrap tests), stores
    bool finite = true;
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int d = 0; d < D; ++d) finite = finite && isfinite(F[j][d]);
    if (!finite) atomicOr(&a.cnt[c].err, kErrNan);
    if (a.frc) {
#pragma unroll
      for (int d = 0; d < D; ++d)
        *reinterpret_cast<double2 *>(a.frc + d * SS + s0) =
            make_double2(static_cast<double>(F[0][d]), static_cast<double>(F[1][d]));
    }
    if (tbits) {
#pragma unroll
      for (int d = 0; d < D; ++d) *reinterpret_cast<float2 *>(a.facc + d * SS + s0) = make_float2(0.0f, 0.0f);
    }
    if (a.integrate) {
      bool inside = true;
      float4 pn[2];
      double xo[2][D];
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const float temp = a.heun ? 0.5f * C.temp_f[j] : C.temp_f[j];
        // 2D: z carries the packed list reference to the next record
        pn[j] = make_float4(0.0f, 0.0f, D == 2 ? pr[j].z : 0.0f, pr[j].w);
        float dj2 = 0.0f;
#pragma unroll
        for (int d = 0; d < D; ++d) {
          const float dxf = temp * F[j][d];
          double xn = xin[j][d] + f2d_exact(dxf);
          const long long xb = __double_as_longlong(xn);
          const long long lb = __double_as_longlong(C.box[d]);
          const bool lo = xb < 0, hi = xb >= lb;  // negative (incl. -0) / at or past L
          if (C.periodic[d]) {
            // the wrap, taken by the few warps with an element that crossed 0 or L (an FP64
            // add predicated into every thread would cost the FP64 pipe on all of them)
            if (__any_sync(__activemask(), lo || hi)) {
              if (lo) xn = (xb & 0x7fffffffffffffffll) ? xn + C.box[d] : 0.0;
              if (__double_as_longlong(xn) >= lb) xn -= C.box[d];
            }
          } else {
            inside = inside && !lo && !hi;
          }
          xo[j][d] = xn;
          const float un = ui[j][d] + dxf;
          pk_set(pn[j], d, un);
          const float dr = un - uref[j][d];
          dj2 += dr * dr;
          st2[j] += dxf * dxf;
        }
        d2 = fmaxf(d2, dj2);
      }
#pragma unroll
      for (int d = 0; d < D; ++d)
        *reinterpret_cast<double2 *>(a.x_out + d * SS + s0) = make_double2(xo[0][d], xo[1][d]);
      a.pk_next[s0] = pn[0];
      a.pk_next[s0 + 1] = pn[1];
      if (!inside) atomicOr(&a.cnt[c].err, kErrBox);
      if (D == 2) {
        // guard with the fixed-point rounding allowed for: trips no later than |u - uref| > skin/2
        const float h = fmaxf(sqrtf(s_half2) - (C.uq_inv[0] + C.uq_inv[1]), 0.0f);
        if (d2 > h * h) atomicOr(&a.skin[c].need, 1);
      } else if (d2 > s_half2) {
        atomicOr(&a.skin[c].need, 1);
      }
      if (a.vel) {
#pragma unroll
        for (int d = 0; d < D; ++d) {
          double v[2];
#pragma unroll
          for (int j = 0; j < 2; ++j) {
            const double vj = static_cast<double>(F[j][d] * C.mu_f[j]);
            v[j] = a.heun == 2 ? 0.5 * ((a.vel_prev ? a.vel_prev : a.vel)[d * SS + s0 + j] + vj) : vj;
          }
          *reinterpret_cast<double2 *>(a.vel + d * SS + s0) = make_double2(v[0], v[1]);
        }
      }
    }
  } else if (used && a.integrate) {
    // tombstones: the next records must keep w < 0 too, or the lists of others would see the
    // stale records of two steps ago in the other buffer
    a.pk_next[s0] = make_float4(0.0f, 0.0f, 0.0f, -1.0f);
    a.pk_next[s0 + 1] = make_float4(0.0f, 0.0f, 0.0f, -1.0f);
  }
  __syncwarp();  // every lane has read its touch word
  if (tword != 0u && (tid & 15) == 0) a.ftouch[s0 >> 5] = 0u;
  if (a.integrate) {
    // displacement statistics: warp reductions and shared atomics; the last warp of the block
    // to finish adds the block's values to the colony (no block barrier: warps with short
    // lists do not wait for the others)
    const unsigned dmax = __reduce_max_sync(0xffffffffu, __float_as_uint(d2));
    const float stp0 = sqrtf(st2[0]), stp1 = sqrtf(st2[1]);
    const unsigned smax = __reduce_max_sync(0xffffffffu, __float_as_uint(fmaxf(stp0, stp1)));
    float ssum = stp0 + stp1;
#pragma unroll
    for (int q = 16; q > 0; q >>= 1) ssum += __shfl_xor_sync(0xffffffffu, ssum, q);
    if ((tid & 31) == 0) {
      atomicMax(&s_dmax, dmax);
      atomicMax(&s_smax, smax);
      atomicAdd(&s_ssum, ssum);
      __threadfence_block();
      if (atomicAdd(&s_warps_done, 1) == TILE / 32 - 1) {
        __threadfence_block();
        StatPart &P = a.spart[c * kStatSlots + (blockIdx.x & (kStatSlots - 1))];
        atomicMax(&P.dmax, atomicOr(&s_dmax, 0u));
        if (a.sched) {
          atomicMax(&P.smax, atomicOr(&s_smax, 0u));
          atomicAdd(&P.ssum, atomicAdd(&s_ssum, 0.0f));
        }
      }
    }
  }
}

template <int D, int LAW, int UNROLL, int MINB, int TILE>
void launch_cells_t(const ForceArgs &a, int grid, cudaStream_t s) {
  constexpr int bytes = (TILE / 32) * pair_smem_warp<D, pair_seg<D, MINB, TILE>()>();
  static bool attr_set = false;  // per instantiation; the attribute is per function
  if (!attr_set) {
    cudaFuncSetAttribute(k_force_cells<D, LAW, UNROLL, MINB, TILE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         bytes);
    attr_set = true;
  }
  k_force_cells<D, LAW, UNROLL, MINB, TILE><<<grid, TILE, bytes, s>>>(a);
}

// MINB is the CTAs per SM at 256 threads; 128-thread blocks keep its threads per SM (hence the
// register budget per thread), 512-thread blocks take at most as many threads per SM
template <int D, int LAW, int UNROLL, int MINB>
void launch_cells(const ForceArgs &a, int grid, int block, cudaStream_t s) {
  if (block == 128)
    launch_cells_t<D, LAW, UNROLL, 2 * MINB, 128>(a, grid, s);
  else if (block == 512)
    launch_cells_t<D, LAW, UNROLL, (MINB / 2 > 0 ? MINB / 2 : 1), 512>(a, grid, s);
  else
    launch_cells_t<D, LAW, UNROLL, MINB, 256>(a, grid, s);
}

template <int D, int LAW>
void launch_list_dl(const ForceArgs &a, int grid, int variant, int block, cudaStream_t s) {
  // cell-major slots, one thread per cell, the warp's list entries flattened; variants
  // (chunks of 32 entries in flight per warp, CTAs per SM at 256 threads): 0 (4, 3), 1 (2, 3),
  // 2 (1, 3), 3 (1, 4); block: 128, 256 or 512 threads (cells per block). The reference's
  // soft-core well is compiled in the default variant only.
  if (LAW == CIL_FORCE_SC || variant == 0) {
    launch_cells<D, LAW, 4, 3>(a, grid, block, s);
  } else if constexpr (LAW != CIL_FORCE_SC) {
    if (variant == 1) {
      launch_cells<D, LAW, 2, 3>(a, grid, block, s);
    } else if (variant == 2) {
      launch_cells<D, LAW, 1, 3>(a, grid, block, s);
    } else {
      launch_cells<D, LAW, 1, 4>(a, grid, block, s);
    }
  }
}

template <int D>
void launch_list_d(const ForceArgs &a, int law, int grid, int variant, int block, cudaStream_t s) {
  switch (law) {
    case CIL_FORCE_LJ_WCA:
      launch_list_dl<D, CIL_FORCE_LJ_WCA>(a, grid, variant, block, s);
      break;
    case CIL_FORCE_SOFTCORE:
      launch_list_dl<D, CIL_FORCE_SOFTCORE>(a, grid, variant, block, s);
      break;
    case CIL_FORCE_SC:
      launch_list_dl<D, CIL_FORCE_SC>(a, grid, variant, block, s);
      break;
    default:
      launch_list_dl<D, CIL_FORCE_HERTZ>(a, grid, variant, block, s);
      break;
  }
}

template <int D>
constexpr size_t mixed_smem_bytes() {
  return sizeof(int) * ((D == 2 ? 9 : 27) * kTile * 2 + kTile + 1 + kTile) + sizeof(float) * (2 * D * kTile + kTile);
}

template <int D, int LAW>
void launch_dl(const ForceArgs &a, int prec, int grid, cudaStream_t s) {
  if (prec == CIL_PREC_FP64) {
    k_force_fp64<D, LAW><<<grid, kTile, 0, s>>>(a);
  } else {
    constexpr size_t bytes = mixed_smem_bytes<D>();
    static bool attr_set = false;  // per instantiation; the attribute is per function
    if (!attr_set) {
      cudaFuncSetAttribute(k_force_mixed<D, LAW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(bytes));
      attr_set = true;
    }
    k_force_mixed<D, LAW><<<grid, kTile, bytes, s>>>(a);
  }
}

template <int D>
void launch_d(const ForceArgs &a, int law, int prec, int grid, cudaStream_t s) {
  switch (law) {
    case CIL_FORCE_LJ_WCA:
      launch_dl<D, CIL_FORCE_LJ_WCA>(a, prec, grid, s);
      break;
    case CIL_FORCE_SOFTCORE:
      launch_dl<D, CIL_FORCE_SOFTCORE>(a, prec, grid, s);
      break;
    case CIL_FORCE_SC:
      launch_dl<D, CIL_FORCE_SC>(a, prec, grid, s);
      break;
    default:
      launch_dl<D, CIL_FORCE_HERTZ>(a, prec, grid, s);
      break;
  }
}

}  // namespace

// This file is compiled twice: with CIL_FORCE_DIM=3 it holds the 3D kernels alone, otherwise
// the 2D kernels and the dispatch (two translation units that build in parallel).
#if defined(CIL_FORCE_DIM) && CIL_FORCE_DIM == 3
void launch_force_list_3d(const ForceArgs &a, int law, int grid, int variant, int block, cudaStream_t s) {
  launch_list_d<3>(a, law, grid, variant, block, s);
}

void launch_force_3d(const ForceArgs &a, int law, int prec, int grid, cudaStream_t s) {
  launch_d<3>(a, law, prec, grid, s);
}
#else
void launch_force_list_3d(const ForceArgs &a, int law, int grid, int variant, int block, cudaStream_t s);
void launch_force_3d(const ForceArgs &a, int law, int prec, int grid, cudaStream_t s);

void launch_force_list(const ForceArgs &a, int dim, int law, int grid, int variant, int block, cudaStream_t s) {
  if (dim == 2)
    launch_list_d<2>(a, law, grid, variant, block, s);
  else
    launch_force_list_3d(a, law, grid, variant, block, s);
}

void launch_force(const ForceArgs &a, int dim, int law, int prec, int grid, int block, cudaStream_t s) {
  (void)block;
  if (dim == 2)
    launch_d<2>(a, law, prec, grid, s);
  else
    launch_force_3d(a, law, prec, grid, s);
}
#endif

}  // namespace cil
