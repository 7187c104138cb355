// Reverse-mode twins of the forward kernels (sm_103a): each takes the
// cotangent of its forward call's output and accumulates (+=) the
// cotangents of the inputs, as the exact transpose of the linearisation of
// the forward call's discrete arithmetic.  The piecewise choices (triangle,
// Powell-Sabin sub-triangle) are held fixed, as in any derivative of a
// piecewise-smooth map.  Scatter into shared records (coefficients, jets,
// SH coefficients) uses FP64 atomics, so sums may differ in the last bits
// between runs.  No counterpart in the reference, which has no derivatives.
#include <cuda_runtime.h>

#include "cmm_internal.h"
#include "device_common.cuh"

namespace cmm {

using namespace dev;

namespace {

constexpr int kBlock = 128;

// Submap coefficient records and their cotangent buffers, by value.
struct AdjPtrs {
  const double* c[kAdjMaxSubmaps];
  double* g[kAdjMaxSubmaps];
};

__device__ __forceinline__ void add_pick(double* bb, int i, double v) {
  if (i == 0) bb[0] += v;
  else if (i == 1) bb[1] += v;
  else bb[2] += v;
}

// ----------------------------------------------------------- assemble
// grad_coeffs (nt, 64) -> grad_jets (3,4,nv) += A^T grad (ncomp = 3).
__global__ void __launch_bounds__(kBlock) assemble_bwd_kernel(MeshView m, const double* __restrict__ gc,
                                                              double* __restrict__ gj) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m.nt) return;
  const int nv = m.nv, nt = m.nt;
  const int4 tv = m.tri_v[t];
  const int vid[3] = {tv.x, tv.y, tv.z};
  const double* A = m.tri_asm + t;
  const int corner[9] = {0, 0, 0, 1, 1, 1, 2, 2, 2};
  double e[9];
#pragma unroll
  for (int j = 0; j < 9; ++j) e[j] = __ldg(A + (int64_t)(36 + j) * nt);
  const double* g = gc + (int64_t)t * kCoeffStride3;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    double c[19];
#pragma unroll
    for (int o = 0; o < 19; ++o) c[o] = g[3 * o + k];
    // c12..c18 are combinations of c3..c11
    c[3] += e[0] * c[12];
    c[8] += e[1] * c[12];
    c[6] += e[2] * c[13];
    c[11] += e[3] * c[13];
    c[9] += e[5] * c[14];
    c[5] += e[4] * c[14];
    c[4] += e[0] * c[15];
    c[7] += e[1] * c[15];
    c[7] += e[2] * c[16];
    c[10] += e[3] * c[16];
    c[4] += e[4] * c[17];
    c[10] += e[5] * c[17];
    c[4] += e[6] * c[18];
    c[7] += e[7] * c[18];
    c[10] += e[8] * c[18];
    double fb[3] = {c[0], c[1], c[2]};
#pragma unroll
    for (int o = 0; o < 9; ++o) {
      const int v = vid[corner[o]];
      const double a0 = __ldg(A + (int64_t)(4 * o) * nt), a1 = __ldg(A + (int64_t)(4 * o + 1) * nt),
                   a2 = __ldg(A + (int64_t)(4 * o + 2) * nt), a3 = __ldg(A + (int64_t)(4 * o + 3) * nt);
      const double cb = c[3 + o];
      atomicAdd(gj + (int64_t)(0 * 4 + 1 + k) * nv + v, a0 * cb);
      atomicAdd(gj + (int64_t)(1 * 4 + 1 + k) * nv + v, a1 * cb);
      atomicAdd(gj + (int64_t)(2 * 4 + 1 + k) * nv + v, a2 * cb);
      fb[corner[o]] -= a3 * cb;
    }
#pragma unroll
    for (int v = 0; v < 3; ++v) atomicAdd(gj + (int64_t)(k * 4) * nv + vid[v], fb[v]);
  }
}

// ------------------------------------------------------------ compose
// Forward pass storing the input point of every submap: work[(s n + i) 3].
__global__ void __launch_bounds__(kBlock) compose_points_kernel(MeshView m, AdjPtrs ap,
                                                                int S, const double* __restrict__ q, int64_t n,
                                                                double* __restrict__ work) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double p[3] = {q[3 * i], q[3 * i + 1], q[3 * i + 2]};
    for (int s = S - 1; s >= 0; --s) {
      double* w = work + 3 * ((int64_t)s * n + i);
      w[0] = p[0];
      w[1] = p[1];
      w[2] = p[2];
      const int t = locate_row(m, p[0], p[1], p[2]);
      double Lr[13];
      load_loc(m, t, Lr);
      const Bcc b = bcc_of(Lr, p[0], p[1], p[2]);
      const Split sp = split_of(b);
      const Gam g = gamma_of(Lr, b, sp);
      Ords<3> o;
      load_ords<3>(ap.c[s] + (int64_t)t * kCoeffStride3, sp, o);
      double P[3];
      sbb<3>(o, g, P);
      const double inv_n = rsqrt(P[0] * P[0] + P[1] * P[1] + P[2] * P[2]);
      p[0] = P[0] * inv_n;
      p[1] = P[1] * inv_n;
      p[2] = P[2] * inv_n;
    }
  }
}

// Reverse pass: cotangent of the composite's output -> cotangents of every
// submap's coefficient records (scatter) and of the query points.
__global__ void __launch_bounds__(kBlock) compose_bwd_kernel(MeshView m, AdjPtrs ap, int S, int64_t n,
                                                             const double* __restrict__ work,
                                                             const double* __restrict__ gout,
                                                             double* __restrict__ gq) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double lam[3] = {gout[3 * i], gout[3 * i + 1], gout[3 * i + 2]};
    for (int s = 0; s < S; ++s) {
      const double* p = work + 3 * ((int64_t)s * n + i);
      const int t = locate_row(m, p[0], p[1], p[2]);
      double Lr[13];
      load_loc(m, t, Lr);
      const Bcc b = bcc_of(Lr, p[0], p[1], p[2]);
      const Split sp = split_of(b);
      const Gam g = gamma_of(Lr, b, sp);
      Ords<3> o;
      load_ords<3>(ap.c[s] + (int64_t)t * kCoeffStride3, sp, o);
      double P[3];
      sbb<3>(o, g, P);
      const double inv_n = rsqrt(P[0] * P[0] + P[1] * P[1] + P[2] * P[2]);
      const double sN[3] = {P[0] * inv_n, P[1] * inv_n, P[2] * inv_n};
      // normalisation: d(P/|P|) = (I - sN sN^T) dP / |P| (symmetric)
      const double sl = sN[0] * lam[0] + sN[1] * lam[1] + sN[2] * lam[2];
      double Pb[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) Pb[c] = (lam[c] - sN[c] * sl) * inv_n;
      // ordinates: P_c = sum_k B_k o_kc
      const double B[6] = {g.V * g.V, g.E * g.E, g.C * g.C, 2 * g.V * g.E, 2 * g.E * g.C, 2 * g.V * g.C};
      const int* id = kSplitOrd[sp.lo][sp.hi];
      double* gr = ap.g[s] + (int64_t)t * kCoeffStride3;
#pragma unroll
      for (int k = 0; k < 6; ++k)
#pragma unroll
        for (int c = 0; c < 3; ++c) atomicAdd(gr + 3 * id[k] + c, B[k] * Pb[c]);
      // sub-triangle barycentrics
      double Vb = 0.0, Eb = 0.0, Cb = 0.0;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        Vb += Pb[c] * 2 * (g.V * o.c[0][c] + g.E * o.c[3][c] + g.C * o.c[5][c]);
        Eb += Pb[c] * 2 * (g.E * o.c[1][c] + g.V * o.c[3][c] + g.C * o.c[4][c]);
        Cb += Pb[c] * 2 * (g.C * o.c[2][c] + g.E * o.c[4][c] + g.V * o.c[5][c]);
      }
      const double en = edge_norm(Lr, sp.hi, sp.mid);
      double bb[3] = {0.0, 0.0, 0.0};
      add_pick(bb, sp.hi, Vb);
      add_pick(bb, sp.mid, -Vb + en * Eb);
      add_pick(bb, sp.lo, -en * Eb + Lr[9] * Cb);
      // b = Minv p
      lam[0] = Lr[0] * bb[0] + Lr[3] * bb[1] + Lr[6] * bb[2];
      lam[1] = Lr[1] * bb[0] + Lr[4] * bb[1] + Lr[7] * bb[2];
      lam[2] = Lr[2] * bb[0] + Lr[5] * bb[1] + Lr[8] * bb[2];
    }
    if (gq) {
      gq[3 * i] += lam[0];
      gq[3 * i + 1] += lam[1];
      gq[3 * i + 2] += lam[2];
    }
  }
}

// ---------------------------------------------------------- vorticity
// grad_X = omega_bar * (grad omega0 + 2 Omega grad cos(theta)); grad omega0
// = -X x (iL omega0)(X) with the three series dsh = iL_x, iL_y, iL_z of
// the initial series (|X| = 1), evaluated together.
__global__ void __launch_bounds__(kBlock) vorticity_bwd_x_kernel(MeshView vm, const double* __restrict__ dsh,
                                                                 int lmax, double rot,
                                                                 const double* __restrict__ X, int64_t Q,
                                                                 const double* __restrict__ gw,
                                                                 double* __restrict__ gX) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Q;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double x = X[3 * i], y = X[3 * i + 1], z = X[3 * i + 2];
    const double wb = gw[i];
    double G[3] = {0.0, 0.0, 0.0};
    if (dsh) {
      double Lv[3];
      sh_series_n<3>(vm, dsh, lmax, sh_point(x, y, z), Lv);
      // -X x (Lx, Ly, Lz)
      G[0] = -(y * Lv[2] - z * Lv[1]);
      G[1] = -(z * Lv[0] - x * Lv[2]);
      G[2] = -(x * Lv[1] - y * Lv[0]);
    }
    // cos(theta) = z / |X|
    const double r2 = x * x + y * y + z * z, r = sqrt(r2);
    G[0] += 2 * rot * (-z * x / r2) / r;
    G[1] += 2 * rot * (-z * y / r2) / r;
    G[2] += 2 * rot * (1.0 - z * z / r2) / r;
    gX[3 * i] += wb * G[0];
    gX[3 * i + 1] += wb * G[1];
    gX[3 * i + 2] += wb * G[2];
  }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  return v;
}

// grad_sh[l][l+-m] += sum_i omega_bar_i Y(X_i): one point per thread, each
// basis value summed over the warp by shuffles, the warp sums gathered in
// shared memory, one global atomic per coefficient per block.
__global__ void __launch_bounds__(256) vorticity_bwd_sh_kernel(MeshView vm, int lmax,
                                                               const double* __restrict__ X, int64_t Q,
                                                               const double* __restrict__ gw,
                                                               double* __restrict__ gsh) {
  extern __shared__ double acc[];   // (lmax+1) x (2 lmax + 1)
  const int w = 2 * lmax + 1;
  const int K = (lmax + 1) * w;
  const int T = kShTableMax + 1;
  for (int k = threadIdx.x; k < K; k += blockDim.x) acc[k] = 0.0;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < Q; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = base + threadIdx.x;
    double wb = 0.0;
    ShPoint pt{1.0, 0.0, 1.0, 0.0};
    if (i < Q) {
      wb = gw[i];
      pt = sh_point(X[3 * i], X[3 * i + 1], X[3 * i + 2]);
    }
    double pmm = 0.28209479177387814, cm = 1.0, sm = 0.0;
    for (int m = 0; m <= lmax; ++m) {
      if (m > 0) {
        pmm = -pmm * __ldg(vm.sh_fm + m) * pt.st;
        const double c2 = cm * pt.cp - sm * pt.sp;
        sm = sm * pt.cp + cm * pt.sp;
        cm = c2;
      }
      const double* ab = vm.sh_ab + 2 * (int64_t)m * T;
      double p1 = 0.0, p = pmm;
      for (int l = m; l <= lmax; ++l) {
        if (l == m + 1) {
          p1 = p;
          p = __ldg(ab + 2 * l) * pt.ct * pmm;
        } else if (l > m + 1) {
          const double pn = __ldg(ab + 2 * l) * (pt.ct * p - __ldg(ab + 2 * l + 1) * p1);
          p1 = p;
          p = pn;
        }
        if (m == 0) {
          const double v = warp_sum(wb * p);
          if (lane == 0) atomicAdd(acc + l * w + l, v);
        } else {
          const double f = wb * 1.4142135623730951 * p;
          const double vc = warp_sum(f * cm), vs = warp_sum(f * sm);
          if (lane == 0) {
            atomicAdd(acc + l * w + l + m, vc);
            atomicAdd(acc + l * w + l - m, vs);
          }
        }
      }
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < K; k += blockDim.x)
    if (acc[k] != 0.0) atomicAdd(gsh + k, acc[k]);
}

// The same sums for lmax <= kShTiledMax without warp shuffles: each warp
// takes 32 points at a time, stages their weighted basis values of one order
// m in shared memory (one row per point), and lane v then sums column v
// over the 32 points into the warp's own coefficient accumulators; the
// block's warps are added at the end, one global atomic per coefficient per
// block.  About half the FP64 work of the shuffle form.
constexpr int kShTiledMax = 32;
constexpr int kShTiledWarps = 4;

__global__ void __launch_bounds__(32 * kShTiledWarps) vorticity_bwd_sh_tiled_kernel(
    MeshView vm, int lmax, const double* __restrict__ X, int64_t Q, const double* __restrict__ gw,
    double* __restrict__ gsh) {
  extern __shared__ double sbuf[];
  const int w = 2 * lmax + 1;
  const int K = (lmax + 1) * w;
  const int T = kShTableMax + 1;
  const int ncol = 2 * (lmax + 1) + 1;   // odd row length against bank conflicts
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* stage = sbuf + (int64_t)warp * (32 * ncol + K);
  double* acc = stage + 32 * ncol;
  for (int k = lane; k < K; k += 32) acc[k] = 0.0;
  __syncwarp();
  const int64_t nw = (int64_t)gridDim.x * kShTiledWarps;
  for (int64_t base = ((int64_t)blockIdx.x * kShTiledWarps + warp) * 32; base < Q; base += nw * 32) {
    const int64_t i = base + lane;
    double wb = 0.0;
    ShPoint pt{1.0, 0.0, 1.0, 0.0};
    if (i < Q) {
      wb = gw[i];
      pt = sh_point(X[3 * i], X[3 * i + 1], X[3 * i + 2]);
    }
    double* row = stage + lane * ncol;
    double pmm = 0.28209479177387814, cm = 1.0, sm = 0.0;
    for (int m = 0; m <= lmax; ++m) {
      if (m > 0) {
        pmm = -pmm * __ldg(vm.sh_fm + m) * pt.st;
        const double c2 = cm * pt.cp - sm * pt.sp;
        sm = sm * pt.cp + cm * pt.sp;
        cm = c2;
      }
      const double* ab = vm.sh_ab + 2 * (int64_t)m * T;
      const int nl = lmax - m + 1;
      double p1 = 0.0, p = pmm;
      for (int l = m; l <= lmax; ++l) {
        if (l == m + 1) {
          p1 = p;
          p = __ldg(ab + 2 * l) * pt.ct * pmm;
        } else if (l > m + 1) {
          const double pn = __ldg(ab + 2 * l) * (pt.ct * p - __ldg(ab + 2 * l + 1) * p1);
          p1 = p;
          p = pn;
        }
        if (m == 0) {
          row[l] = wb * p;
        } else {
          const double f = wb * 1.4142135623730951 * p;
          row[l - m] = f * cm;
          row[nl + l - m] = f * sm;
        }
      }
      __syncwarp();
      const int nvals = m == 0 ? nl : 2 * nl;
      for (int v = lane; v < nvals; v += 32) {
        double sum = 0.0;
#pragma unroll 8
        for (int q = 0; q < 32; ++q) sum += stage[q * ncol + v];
        const int j = v < nl ? v : v - nl, l = m + j;
        acc[l * w + l + (v < nl ? m : -m)] += sum;
      }
      __syncwarp();
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < K; k += blockDim.x) {
    double t = 0.0;
    for (int wp = 0; wp < kShTiledWarps; ++wp) t += sbuf[(int64_t)wp * (32 * ncol + K) + 32 * ncol + k];
    if (t != 0.0) atomicAdd(gsh + k, t);
  }
}

// ---------------------------------------------------------- map update
// Gradient of a patch P(gamma(b(p))) at p (fixed sub-triangle): given the
// cotangents (Vb, Eb, Cb) of the sub-triangle barycentrics, pbar += Minv^T
// (dgamma/db)^T (Vb, Eb, Cb).
__device__ __forceinline__ void gamma_to_point(const double* Lr, const Split& sp, double Vb, double Eb,
                                               double Cb, double* pb) {
  const double en = edge_norm(Lr, sp.hi, sp.mid);
  double bb[3] = {0.0, 0.0, 0.0};
  add_pick(bb, sp.hi, Vb);
  add_pick(bb, sp.mid, -Vb + en * Eb);
  add_pick(bb, sp.lo, -en * Eb + Lr[9] * Cb);
  pb[0] += Lr[0] * bb[0] + Lr[3] * bb[1] + Lr[6] * bb[2];
  pb[1] += Lr[1] * bb[0] + Lr[4] * bb[1] + Lr[7] * bb[2];
  pb[2] += Lr[2] * bb[0] + Lr[5] * bb[1] + Lr[8] * bb[2];
}

// (Vb, Eb, Cb) += sum_c Pb_c dP_c/d(V, E, C) for P = sbb(o, g).
__device__ __forceinline__ void patch_gamma_bwd(const Ords<3>& o, const Gam& g, const double* Pb, double& Vb,
                                                double& Eb, double& Cb) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    Vb += Pb[c] * 2 * (g.V * o.c[0][c] + g.E * o.c[3][c] + g.C * o.c[5][c]);
    Eb += Pb[c] * 2 * (g.E * o.c[1][c] + g.V * o.c[3][c] + g.C * o.c[4][c]);
    Cb += Pb[c] * 2 * (g.C * o.c[2][c] + g.E * o.c[4][c] + g.V * o.c[5][c]);
  }
}

__device__ __forceinline__ void scatter_ords(double* rec, const Split& sp, const Gam& g, const double* Pb,
                                             double scale) {
  const double B[6] = {g.V * g.V, g.E * g.E, g.C * g.C, 2 * g.V * g.E, 2 * g.E * g.C, 2 * g.V * g.C};
  const int* id = kSplitOrd[sp.lo][sp.hi];
#pragma unroll
  for (int k = 0; k < 6; ++k)
#pragma unroll
    for (int c = 0; c < 3; ++c) atomicAdd(rec + 3 * id[k] + c, scale * B[k] * Pb[c]);
}

struct VelGrad {
  const double* v[3];   // velocity records (time levels)
  double* g[3];         // their cotangents
};

__device__ __forceinline__ void vel_eval(const MeshView& vm, const VelGrad& vg, int nvs, const double* w,
                                         const double* p, double* V) {
  const int t = latlon_locate(vm, p[0], p[1], p[2]);
  double Lr[13];
  load_loc(vm, t, Lr);
  const Bcc b = bcc_of(Lr, p[0], p[1], p[2]);
  const Split sp = split_of(b);
  const Gam g = gamma_of(Lr, b, sp);
  V[0] = V[1] = V[2] = 0.0;
  for (int l = 0; l < nvs; ++l) {
    Ords<3> o;
    load_ords<3>(vg.v[l] + (int64_t)t * kCoeffStride3, sp, o);
    double P[3];
    sbb<3>(o, g, P);
    V[0] += w[l] * P[0];
    V[1] += w[l] * P[1];
    V[2] += w[l] * P[2];
  }
}

// Velocity V(p) = sum_l w_l P_l(p): pbar += J_V^T vb; records += w_l B vb.
__device__ __forceinline__ void vel_bwd(const MeshView& vm, const VelGrad& vg, int nvs, const double* w,
                                        const double* p, const double* vb, double* pb) {
  const int t = latlon_locate(vm, p[0], p[1], p[2]);
  double Lr[13];
  load_loc(vm, t, Lr);
  const Bcc b = bcc_of(Lr, p[0], p[1], p[2]);
  const Split sp = split_of(b);
  const Gam g = gamma_of(Lr, b, sp);
  double Vb = 0.0, Eb = 0.0, Cb = 0.0;
  for (int l = 0; l < nvs; ++l) {
    Ords<3> o;
    load_ords<3>(vg.v[l] + (int64_t)t * kCoeffStride3, sp, o);
    const double Pb[3] = {w[l] * vb[0], w[l] * vb[1], w[l] * vb[2]};
    patch_gamma_bwd(o, g, Pb, Vb, Eb, Cb);
    scatter_ords(vg.g[l] + (int64_t)t * kCoeffStride3, sp, g, vb, w[l]);
  }
  if (pb) gamma_to_point(Lr, sp, Vb, Eb, Cb, pb);
}

// y -> y / |y|: ybar = (I - s s^T) sbar / |y|
__device__ __forceinline__ void proj_bwd(const double* y, const double* sb, double* yb) {
  const double r = sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
  const double s0 = y[0] / r, s1 = y[1] / r, s2 = y[2] / r;
  const double d = s0 * sb[0] + s1 * sb[1] + s2 * sb[2];
  yb[0] = (sb[0] - s0 * d) / r;
  yb[1] = (sb[1] - s1 * d) / r;
  yb[2] = (sb[2] - s2 * d) / r;
}

__device__ __forceinline__ void proj(const double* y, double* s) {   // as sphere_proj
  const double r = rsqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
  s[0] = y[0] * r;
  s[1] = y[1] * r;
  s[2] = y[2] * r;
}

// Reverse of the backward integrators (scheme 0 Euler, 1 improved Euler,
// 2 RK4; the forward arithmetic of integrate_point) for the stencil points
// (their start points are constants): the foot-point cotangents -> the
// velocity records' cotangents.
__global__ void __launch_bounds__(kBlock) advect_points_bwd_kernel(MeshView mesh, MeshView vm, VelGrad vg,
                                                                   int nvs, TimeWeights tw, int scheme,
                                                                   double dt,
                                                                   const double* __restrict__ s_pts,
                                                                   const double* __restrict__ gsn) {
  const int64_t nv = mesh.nv, n = 4 * nv;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n;
       j += (int64_t)gridDim.x * blockDim.x) {
    const double xb[3] = {gsn[j], gsn[4 * nv + j], gsn[8 * nv + j]};
    if (xb[0] == 0.0 && xb[1] == 0.0 && xb[2] == 0.0) continue;
    const double p0[3] = {s_pts[j], s_pts[4 * nv + j], s_pts[8 * nv + j]};
    const double* w0 = tw.w[0];
    const double* w1 = tw.w[1];
    const double* w2 = tw.w[2];
    const double* w3 = tw.w[3];
    double v1[3], v2[3], v3[3], v4[3], y1[3], y2[3], y3[3], y4[3], s1[3], s2[3], s3[3];
    vel_eval(vm, vg, nvs, w0, p0, v1);
    if (scheme == 0) {
      for (int c = 0; c < 3; ++c) y4[c] = p0[c] - dt * v1[c];
      double yb[3];
      proj_bwd(y4, xb, yb);
      const double v1b[3] = {-dt * yb[0], -dt * yb[1], -dt * yb[2]};
      vel_bwd(vm, vg, nvs, w0, p0, v1b, nullptr);
      continue;
    }
    if (scheme == 1) {
      for (int c = 0; c < 3; ++c) y1[c] = p0[c] - dt * v1[c];
      proj(y1, s1);
      vel_eval(vm, vg, nvs, w1, s1, v2);
      for (int c = 0; c < 3; ++c) y4[c] = p0[c] - (dt / 2) * (v1[c] + v2[c]);
      double yb[3];
      proj_bwd(y4, xb, yb);
      double v1b[3], v2b[3];
      for (int c = 0; c < 3; ++c) v1b[c] = v2b[c] = -(dt / 2) * yb[c];
      double s1b[3] = {0.0, 0.0, 0.0};
      vel_bwd(vm, vg, nvs, w1, s1, v2b, s1b);
      double y1b[3];
      proj_bwd(y1, s1b, y1b);
      for (int c = 0; c < 3; ++c) v1b[c] += -dt * y1b[c];
      vel_bwd(vm, vg, nvs, w0, p0, v1b, nullptr);
      continue;
    }
    for (int c = 0; c < 3; ++c) y1[c] = p0[c] - dt * v1[c] / 2;
    proj(y1, s1);
    vel_eval(vm, vg, nvs, w1, s1, v2);
    for (int c = 0; c < 3; ++c) y2[c] = p0[c] - (dt / 2) * v2[c];
    proj(y2, s2);
    vel_eval(vm, vg, nvs, w2, s2, v3);
    for (int c = 0; c < 3; ++c) y3[c] = p0[c] - dt * v3[c];
    proj(y3, s3);
    vel_eval(vm, vg, nvs, w3, s3, v4);
    for (int c = 0; c < 3; ++c) y4[c] = p0[c] - (dt / 6) * (v1[c] + 2 * v2[c] + 2 * v3[c] + v4[c]);
    double yb[3];
    proj_bwd(y4, xb, yb);
    double v1b[3], v2b[3], v3b[3], v4b[3];
    for (int c = 0; c < 3; ++c) {
      v1b[c] = -(dt / 6) * yb[c];
      v2b[c] = -(dt / 6) * 2 * yb[c];
      v3b[c] = -(dt / 6) * 2 * yb[c];
      v4b[c] = -(dt / 6) * yb[c];
    }
    double sb[3] = {0.0, 0.0, 0.0}, ybb[3];
    vel_bwd(vm, vg, nvs, w3, s3, v4b, sb);
    proj_bwd(y3, sb, ybb);
    for (int c = 0; c < 3; ++c) v3b[c] += -dt * ybb[c];
    sb[0] = sb[1] = sb[2] = 0.0;
    vel_bwd(vm, vg, nvs, w2, s2, v3b, sb);
    proj_bwd(y2, sb, ybb);
    for (int c = 0; c < 3; ++c) v2b[c] += -(dt / 2) * ybb[c];
    sb[0] = sb[1] = sb[2] = 0.0;
    vel_bwd(vm, vg, nvs, w1, s1, v2b, sb);
    proj_bwd(y1, sb, ybb);
    for (int c = 0; c < 3; ++c) v1b[c] += -(dt / 2) * ybb[c];
    vel_bwd(vm, vg, nvs, w0, p0, v1b, nullptr);
  }
}

// Reverse of project_jets_kernel: jet cotangents -> cotangents of the
// stencil foot points (gsn, overwritten) and, with a previous map, of its
// records (gprev +=).  The vertex foot point only selects the previous
// map's patch and carries no derivative.
__global__ void __launch_bounds__(kBlock) project_jets_bwd_kernel(MeshView m, const double* __restrict__ prev,
                                                                  double* __restrict__ gprev,
                                                                  const double* __restrict__ yn,
                                                                  const double* __restrict__ sn,
                                                                  const double* __restrict__ tan, double eps,
                                                                  const double* __restrict__ gj,
                                                                  double* __restrict__ gsn) {
  const int64_t nv = m.nv;
  const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (v >= nv) return;
  double S[4][3];
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int c = 0; c < 3; ++c) S[k][c] = sn[(c * 4 + k) * nv + v];
  int t = 0;
  Split sp{0, 0, 0};
  double Lr[13];
  Ords<3> o;
  Gam gk[4];
  if (prev) {
    const double x = yn[v], y = yn[nv + v], z = yn[2 * nv + v];
    t = locate_row(m, x, y, z);
    load_loc(m, t, Lr);
    sp = split_of(bcc_of(Lr, x, y, z));
    load_ords<3>(prev + (int64_t)t * kCoeffStride3, sp, o);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      gk[k] = gamma_of(Lr, bcc_of(Lr, S[k][0], S[k][1], S[k][2]), sp);
      double P[3];
      sbb<3>(o, gk[k], P);
      S[k][0] = P[0];
      S[k][1] = P[1];
      S[k][2] = P[2];
    }
  }
  double mv[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) mv[c] = (S[0][c] + S[1][c] + S[2][c] + S[3][c]) / 4;
  const double nm = sqrt(mv[0] * mv[0] + mv[1] * mv[1] + mv[2] * mv[2]);
  const double* a1 = tan + 3 * v;
  const double* a2 = tan + 3 * (nv + v);
  // value: jets[c][0] = mv_c / nm
  double jb[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) jb[c] = gj[(c * 4 + 0) * nv + v];
  double mb[3];
  proj_bwd(mv, jb, mb);
  // gradients: jets[c][1+k] = d1_k a1_c + d2_k a2_c
  double d1b[3], d2b[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    double s1 = 0.0, s2 = 0.0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double g = gj[(c * 4 + 1 + k) * nv + v];
      s1 += a1[c] * g;
      s2 += a2[c] * g;
    }
    d1b[k] = s1;
    d2b[k] = s2;
  }
  double Sb[4][3];
  const double f = 1.0 / (4 * eps);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    Sb[0][c] = mb[c] / 4 - f * d1b[c] - f * d2b[c];
    Sb[1][c] = mb[c] / 4 + f * d1b[c] - f * d2b[c];
    Sb[2][c] = mb[c] / 4 - f * d1b[c] + f * d2b[c];
    Sb[3][c] = mb[c] / 4 + f * d1b[c] + f * d2b[c];
  }
  if (prev) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      double Vb = 0.0, Eb = 0.0, Cb = 0.0;
      patch_gamma_bwd(o, gk[k], Sb[k], Vb, Eb, Cb);
      if (gprev) scatter_ords(gprev + (int64_t)t * kCoeffStride3, sp, gk[k], Sb[k], 1.0);
      double pb[3] = {0.0, 0.0, 0.0};
      gamma_to_point(Lr, sp, Vb, Eb, Cb, pb);
      Sb[k][0] = pb[0];
      Sb[k][1] = pb[1];
      Sb[k][2] = pb[2];
    }
  }
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int c = 0; c < 3; ++c) gsn[(c * 4 + k) * nv + v] = Sb[k][c];
}

int check(const char* what) {
  note_launch();
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? CMM_OK : cuda_fail(e, what);
}

}  // namespace

int launch_assemble_bwd(const MeshView& m, const double* gc, double* gj, cudaStream_t s) {
  assemble_bwd_kernel<<<(m.nt + kBlock - 1) / kBlock, kBlock, 0, s>>>(m, gc, gj);
  return check("assemble_bwd_kernel");
}

int launch_compose_bwd(const MeshView& m, const double* const* cs, double* const* gcs, int S,
                       const double* q, int64_t n, const double* gout, double* gq, double* work,
                       cudaStream_t s) {
  if (n == 0) return CMM_OK;
  AdjPtrs ap;
  for (int k = 0; k < S; ++k) {
    ap.c[k] = cs[k];
    ap.g[k] = gcs[k];
  }
  const int g = grid_for(n, kBlock);
  compose_points_kernel<<<g, kBlock, 0, s>>>(m, ap, S, q, n, work);
  int rc = check("compose_points_kernel");
  if (rc) return rc;
  compose_bwd_kernel<<<g, kBlock, 0, s>>>(m, ap, S, n, work, gout, gq);
  return check("compose_bwd_kernel");
}

int launch_advect_project_bwd(const MeshView& mesh, const MeshView& vm, const double* const* vel,
                              double* const* gvel, int nvs, const TimeWeights& tw, int scheme, double dt,
                              const double* s_pts, const double* tan, const double* prev, double* gprev,
                              double eps, const double* gjets, double* work, cudaStream_t s) {
  const int64_t nv = mesh.nv;
  VelPtrs vc{};
  VelGrad vg{};
  for (int l = 0; l < nvs; ++l) {
    vc.p[l] = vel[l];
    vg.v[l] = vel[l];
    vg.g[l] = gvel[l];
  }
  // forward foot points again (work: yn, sn), then the two reverse passes
  int rc = launch_advect_points(mesh, vm, vc, nvs, tw, scheme, dt, s_pts, work, s);
  if (rc) return rc;
  double* gsn = work + 15 * nv;
  project_jets_bwd_kernel<<<(int)((nv + kBlock - 1) / kBlock), kBlock, 0, s>>>(
      mesh, prev, gprev, work, work + 3 * nv, tan, eps, gjets, gsn);
  if ((rc = check("project_jets_bwd_kernel"))) return rc;
  advect_points_bwd_kernel<<<grid_for(4 * nv, kBlock), kBlock, 0, s>>>(mesh, vm, vg, nvs, tw, scheme, dt,
                                                                       s_pts, gsn);
  return check("advect_points_bwd_kernel");
}

int launch_vorticity_bwd(const MeshView& vm, const double* dsh, int lmax, double rot, const double* X,
                         int64_t Q, const double* gw, double* gX, double* gsh, cudaStream_t s) {
  if (lmax > kShTableMax) {
    set_last_error("cmm_vorticity_bwd: lmax must be <= 128");
    return CMM_ERR_UNSUPPORTED;
  }
  if (gX) {
    vorticity_bwd_x_kernel<<<grid_for(Q, kBlock), kBlock, 0, s>>>(vm, dsh, lmax, rot, X, Q, gw, gX);
    int rc = check("vorticity_bwd_x_kernel");
    if (rc) return rc;
  }
  if (gsh && lmax >= 0 && lmax <= kShTiledMax) {
    const int ncol = 2 * (lmax + 1) + 1;
    const size_t smem = sizeof(double) * (size_t)kShTiledWarps *
                        (32 * ncol + (size_t)(lmax + 1) * (2 * lmax + 1));
    cudaError_t e = cudaFuncSetAttribute(vorticity_bwd_sh_tiled_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(vorticity_bwd_sh_tiled_kernel)");
    const int64_t chunks = (Q + 32 * kShTiledWarps - 1) / (32 * kShTiledWarps);
    const int g = (int)(chunks < 2 * 152 ? chunks : 2 * 152);
    vorticity_bwd_sh_tiled_kernel<<<g, 32 * kShTiledWarps, smem, s>>>(vm, lmax, X, Q, gw, gsh);
    return check("vorticity_bwd_sh_tiled_kernel");
  }
  if (gsh && lmax >= 0) {
    const size_t smem = sizeof(double) * (size_t)(lmax + 1) * (2 * lmax + 1);
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(vorticity_bwd_sh_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem);
      if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(vorticity_bwd_sh_kernel)");
    }
    vorticity_bwd_sh_kernel<<<grid_for(Q, 256), 256, smem, s>>>(vm, lmax, X, Q, gw, gsh);
    return check("vorticity_bwd_sh_kernel");
  }
  return CMM_OK;
}

}  // namespace cmm
