// Fused force + integrate kernel: one thread per binned element.
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
// Precision forms:
//   FP64   positions, displacements and force arithmetic in FP64
//   MIXED  displacements from FP32 bin-local coordinates (written by the rebuild) plus the
//          FP32 bin offset, FP32 force law, FP64 accumulation into the element force and
//          FP64 integration and wrap.
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

template <int D, int LAW, int PREC>
__global__ void __launch_bounds__(kTile) k_force(ForceArgs a) {
  const int total = a.tiles_live[a.B];
  for (int t = blockIdx.x; t < total; t += gridDim.x) {
    const int c = colony_of_tile(a.tiles_live, a.B, t);
    const ColonyConst &C = a.col[c];
    const int s = C.slot_base + (t - a.tiles_live[c]) * kTile + threadIdx.x;
    const int nlive = a.cnt[c].nlive;
    if (s >= C.slot_base + nlive) continue;

    const size_t SS = a.SS;
    const int e = a.eid[s];
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
      } else {
        const double r = sqrt(r2);
        double rest = C.rest0;
        if (C.divide) {
          const int t0 = a.t0[g], tsw = a.tsw[g];
          const int span = tsw - t0;
          double frac = span > 0 ? static_cast<double>(a.ts - t0) / static_cast<double>(span) : 1.0;
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
      const uint32_t id = static_cast<uint32_t>(C.noise_per_cell ? g : e);
      const u32x4 r = philox4x32_10(id, static_cast<uint32_t>(a.ts), kRngNoise, 0u, a.seed_lo, a.seed_hi);
      float n[4];
      box_muller(r.v[0], r.v[1], n[0], n[1]);
      box_muller(r.v[2], r.v[3], n[2], n[3]);
#pragma unroll
      for (int d = 0; d < D; ++d) F[d] += C.zeta[j] * (C.noise_amp * static_cast<double>(n[d]));
    }

    // ---- pair forces
    int bi[D];
    bin_coords<D>(C, xi, bi);
    if (C.single_bin) {
      // one bin: all elements, minimum image as BoundingBox::distance (Utils.hpp:536-544)
      const double eps = C.epsilon, rcs = C.rcut_scale;
      for (int tt = C.slot_base; tt < C.slot_base + nlive; ++tt) {
        const int ej = a.eid[tt];
        if ((ej >> 1) == g) continue;
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
        if (pair_force<LAW, double>(r2, si, a.sig[tt], eps, rcs, f0)) {
#pragma unroll
          for (int d = 0; d < D; ++d) F[d] += f0 * dx[d];
        }
      }
    } else if (PREC == CIL_PREC_FP64) {
      const double eps = C.epsilon, rcs = C.rcut_scale;
      int o[3] = {-1, -1, -1};
      for (o[0] = -1; o[0] <= 1; ++o[0])
        for (o[1] = -1; o[1] <= 1; ++o[1])
          for (o[2] = (D == 3 ? -1 : 0); o[2] <= (D == 3 ? 1 : 0); ++o[2]) {
            int nb[D];
            double shift[D];
            if (!neighbor_bin<D>(C, bi, o, nb, shift)) continue;
            const int2 r = a.range[C.bin_base + bin_id<D>(C, nb)];
            for (int tt = r.x; tt < r.y; ++tt) {
              const int ej = __ldg(a.eid + tt);
              if ((ej >> 1) == g) continue;
              double dx[D];
              double r2 = 0.0;
#pragma unroll
              for (int d = 0; d < D; ++d) {
                dx[d] = (__ldg(a.x_in + d * SS + tt) + shift[d]) - xi[d];
                r2 += dx[d] * dx[d];
              }
              double f0;
              if (pair_force<LAW, double>(r2, si, __ldg(a.sig + tt), eps, rcs, f0)) {
#pragma unroll
                for (int d = 0; d < D; ++d) F[d] += f0 * dx[d];
              }
            }
          }
    } else {
      const float eps = static_cast<float>(C.epsilon), rcs = static_cast<float>(C.rcut_scale);
      float ui[D];
#pragma unroll
      for (int d = 0; d < D; ++d) ui[d] = a.u[d * SS + s];
      const float sif = a.sigf[s];
      float Fp[D];
#pragma unroll
      for (int d = 0; d < D; ++d) Fp[d] = 0.0f;
      int o[3] = {-1, -1, -1};
      for (o[0] = -1; o[0] <= 1; ++o[0])
        for (o[1] = -1; o[1] <= 1; ++o[1])
          for (o[2] = (D == 3 ? -1 : 0); o[2] <= (D == 3 ? 1 : 0); ++o[2]) {
            int nb[D];
            double shift[D];
            if (!neighbor_bin<D>(C, bi, o, nb, shift)) continue;
            float off[D];
#pragma unroll
            for (int d = 0; d < D; ++d) off[d] = static_cast<float>(o[d]) * C.bwf[d] - ui[d];
            const int2 r = a.range[C.bin_base + bin_id<D>(C, nb)];
            for (int tt = r.x; tt < r.y; ++tt) {
              const int ej = __ldg(a.eid + tt);
              if ((ej >> 1) == g) continue;
              float dx[D];
              float r2 = 0.0f;
#pragma unroll
              for (int d = 0; d < D; ++d) {
                dx[d] = __ldg(a.u + d * SS + tt) + off[d];
                r2 += dx[d] * dx[d];
              }
              float f0;
              if (pair_force<LAW, float>(r2, sif, __ldg(a.sigf + tt), eps, rcs, f0)) {
#pragma unroll
                for (int d = 0; d < D; ++d) Fp[d] += f0 * dx[d];
              }
            }
          }
#pragma unroll
      for (int d = 0; d < D; ++d) F[d] += static_cast<double>(Fp[d]);
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
      const double temp = C.temp[j];
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
        for (int d = 0; d < D; ++d) a.vel[d * SS + s] = F[d] * C.mu_eff[j];
      }
    }
  }
}

template <int D, int LAW>
void launch_dl(const ForceArgs &a, int prec, int grid, int block, cudaStream_t s) {
  (void)block;
  if (prec == CIL_PREC_FP64)
    k_force<D, LAW, CIL_PREC_FP64><<<grid, kTile, 0, s>>>(a);
  else
    k_force<D, LAW, CIL_PREC_MIXED><<<grid, kTile, 0, s>>>(a);
}

template <int D>
void launch_d(const ForceArgs &a, int law, int prec, int grid, int block, cudaStream_t s) {
  switch (law) {
    case CIL_FORCE_LJ_WCA:
      launch_dl<D, CIL_FORCE_LJ_WCA>(a, prec, grid, block, s);
      break;
    case CIL_FORCE_SOFTCORE:
      launch_dl<D, CIL_FORCE_SOFTCORE>(a, prec, grid, block, s);
      break;
    default:
      launch_dl<D, CIL_FORCE_HERTZ>(a, prec, grid, block, s);
      break;
  }
}

}  // namespace

void launch_force(const ForceArgs &a, int dim, int law, int prec, int grid, int block,
                  cudaStream_t s) {
  if (dim == 2)
    launch_d<2>(a, law, prec, grid, block, s);
  else
    launch_d<3>(a, law, prec, grid, block, s);
}

}  // namespace cil
