// MWSS spherical-harmonic transforms and the vorticity -> velocity-jet
// pipeline (sm_103a, FP64).
//
// Forward (inv_Laplacian, cmm_s2/core/spherical_harmonic_tools.py:14-19):
//   1. rfft along each of the L+1 rings (cuFFT D2Z), scaled by pi/L;
//   2. per m, the theta-torus extension F_m(2pi - theta) = (-1)^m F_m(theta)
//      and its trigonometric interpolant (Nyquist term split evenly) are
//      resampled on 2L+1 rings theta'_j = pi j / 2L (cuFFT Z2Z 2L forward,
//      zero padding, Z2Z 4L inverse);
//   3. Legendre analysis with Clenshaw-Curtis weights in cos(theta), exact
//      for the degree <= 2L-1 products: f_lm = sum_j w_j F'_m(j) Pbar_lm(j).
// Inverse (pyssht.inverse in project_stream, :84-91): Legendre synthesis on
// the L+1 rings, then inverse real FFTs (cuFFT Z2D).
// Pbar_lm are orthonormal with the Condon-Shortley phase and come from the
// three-term recurrence in l run on the fly (FP64); rings theta and
// pi - theta are processed together since Pbar_lm(pi - theta) =
// (-1)^(l+m) Pbar_lm(theta).  In CMM_SHT_SPLIT_BF16 mode both Legendre
// contractions (forward analysis, 12-field synthesis) run instead on the
// tensor cores from precomputed split-bf16 tables (sht_tc.cu).
// Coefficient layout on the device: alm[m][l] complex (double2), m-major,
// m <= l < L, entries with l < m unused and zero.
#include <cuda_runtime.h>
#include <cufft.h>

#include <cmath>
#include <memory>
#include <vector>

#include "cmm_internal.h"

namespace cmm {

namespace {

constexpr int kFields = 12;   // 3 velocity components + 3x3 gradients
constexpr int kSynthBlock = 64;
constexpr int kLChunk = 32;

__device__ __forceinline__ double2 cmul(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 cmul(float2 a, double s) {
  return make_float2(a.x * (float)s, a.y * (float)s);
}

// ----------------------------------------------------------------- forward
// C = double2 (FP64 form) or float2 (ring FFTs of the split-BF16 form).
// F (L+1, L+1) ring spectra -> torus columns G (2L, L): G[t][m].
template <typename C>
__global__ void torus_kernel(const C* __restrict__ F, int L, C* __restrict__ G) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  const int t = blockIdx.y;
  if (m >= L || t >= 2 * L) return;
  const double s = M_PI / L;
  C v;
  if (t <= L) {
    v = F[(int64_t)t * (L + 1) + m];
  } else {
    v = F[(int64_t)(2 * L - t) * (L + 1) + m];
    if (m & 1) {
      v.x = -v.x;
      v.y = -v.y;
    }
  }
  G[(int64_t)t * L + m] = cmul(v, s);
}

// Torus spectrum Gh (2L, L) -> zero-padded H (4L, L), Nyquist split.
template <typename C>
__global__ void pad_kernel(const C* __restrict__ Gh, int L, C* __restrict__ H) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y;  // 0..4L-1
  if (m >= L || k >= 4 * L) return;
  const double s = 1.0 / (2 * L);
  C v;
  v.x = 0;
  v.y = 0;
  if (k < L) {
    v = Gh[(int64_t)k * L + m];
  } else if (k == L || k == 3 * L) {
    v = cmul(Gh[(int64_t)L * L + m], 0.5);
  } else if (k > 3 * L) {
    v = Gh[(int64_t)(k - 2 * L) * L + m];
  }
  H[(int64_t)k * L + m] = cmul(v, s);
}

// The FP64 form keeps the torus and padded spectra order-major, G[m][t]
// (L, 2L) and H[m][k] (L, 4L), so that cuFFT transforms L contiguous rows
// (the strided column transforms of the layout above run a few blocks at
// small L).  Same values as torus_kernel / pad_kernel.
__global__ void torus_t_kernel(const double2* __restrict__ F, int L, double2* __restrict__ G) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  const int t = blockIdx.y;
  if (m >= L || t >= 2 * L) return;
  const double s = M_PI / L;
  double2 v;
  if (t <= L) {
    v = F[(int64_t)t * (L + 1) + m];
  } else {
    v = F[(int64_t)(2 * L - t) * (L + 1) + m];
    if (m & 1) {
      v.x = -v.x;
      v.y = -v.y;
    }
  }
  G[(int64_t)m * 2 * L + t] = cmul(v, s);
}

__global__ void pad_t_kernel(const double2* __restrict__ Gh, int L, double2* __restrict__ H) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;  // 0..4L-1
  const int m = blockIdx.y;
  if (k >= 4 * L || m >= L) return;
  const double s = 1.0 / (2 * L);
  const double2* g = Gh + (int64_t)m * 2 * L;
  double2 v = make_double2(0.0, 0.0);
  if (k < L) {
    v = g[k];
  } else if (k == L || k == 3 * L) {
    v = cmul(g[L], 0.5);
  } else if (k > 3 * L) {
    v = g[k - 2 * L];
  }
  H[(int64_t)m * 4 * L + k] = cmul(v, s);
}

// Zero the m = L column of nrows spectra rows of length L+1 (an
// out-of-place C2R transform may overwrite its input).
__global__ void zero_nyquist_kernel(float2* __restrict__ S, int L, int nrows) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < nrows) S[(int64_t)r * (L + 1) + L] = make_float2(0.f, 0.f);
}

// FP64 samples -> FP32 (input of the split form's ring FFT).
__global__ void to_float_kernel(const double* __restrict__ a, int64_t n, float* __restrict__ b) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

__global__ void to_double_kernel(const float* __restrict__ a, int64_t n, double* __restrict__ b) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = (double)a[i];
}

// Legendre analysis: one block per m; ring pairs (j, 2L-j) of the fine grid
// with the quadrature weights folded in.  fine (L, 4L) order-major: rings
// 0..2L of each order used.
__global__ void __launch_bounds__(256) analysis_kernel(const double2* __restrict__ fine, int L,
                                                       const double* __restrict__ w,
                                                       const double* __restrict__ ct,
                                                       const double* __restrict__ pmm,
                                                       const double* __restrict__ ra,
                                                       const double* __restrict__ rb,
                                                       double2* __restrict__ alm) {
  const int m = blockIdx.x;
  const int npair = L + 1;  // j = 0..L (j = L is the equator, unpaired)
  constexpr int R = 8;      // ring pairs per thread (up to 2048 pairs)
  double2 E[R], O[R];
  double x[R], p0[R], p1[R];
  int nr = 0;
  for (int r = 0; r < R; ++r) {
    const int j = threadIdx.x + r * blockDim.x;
    if (j < npair) {
      const double2 a = fine[(int64_t)m * 4 * L + j];
      double2 e, o;
      if (j < L) {
        const double2 b = fine[(int64_t)m * 4 * L + 2 * L - j];
        e = make_double2(a.x + b.x, a.y + b.y);
        o = make_double2(a.x - b.x, a.y - b.y);
      } else {
        e = a;
        o = make_double2(0.0, 0.0);
      }
      E[r] = cmul(e, w[j]);
      O[r] = cmul(o, w[j]);
      x[r] = ct[j];
      p0[r] = pmm[(int64_t)m * (2 * L + 1) + j];  // Pbar_mm
      p1[r] = 0.0;
      nr = r + 1;
    } else {
      E[r] = O[r] = make_double2(0.0, 0.0);
      x[r] = p0[r] = p1[r] = 0.0;
    }
  }
  __shared__ double2 red[kLChunk][8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int l0 = m; l0 < L; l0 += kLChunk) {
    double2 acc[kLChunk];
#pragma unroll
    for (int q = 0; q < kLChunk; ++q) acc[q] = make_double2(0.0, 0.0);
#pragma unroll
    for (int q = 0; q < kLChunk; ++q) {
      const int l = l0 + q;
      if (l < L) {
        const bool even = ((l - m) & 1) == 0;
        double a = 0.0, b = 0.0;
        if (l > m) {
          a = ra[(int64_t)m * L + l];
          b = rb[(int64_t)m * L + l];
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
          if (r < nr) {
            double P;
            if (l == m) {
              P = p0[r];
            } else if (l == m + 1) {
              P = a * x[r] * p0[r];
              p1[r] = p0[r];
              p0[r] = P;
            } else {
              P = a * (x[r] * p0[r] - b * p1[r]);
              p1[r] = p0[r];
              p0[r] = P;
            }
            const double2 v = even ? E[r] : O[r];
            acc[q].x += P * v.x;
            acc[q].y += P * v.y;
          }
        }
      }
    }
    // block reduction of the chunk
#pragma unroll
    for (int q = 0; q < kLChunk; ++q) {
      double vx = acc[q].x, vy = acc[q].y;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        vx += __shfl_down_sync(0xffffffffu, vx, off);
        vy += __shfl_down_sync(0xffffffffu, vy, off);
      }
      if (lane == 0) red[q][warp] = make_double2(vx, vy);
    }
    __syncthreads();
    if (threadIdx.x < kLChunk) {
      const int q = threadIdx.x, l = l0 + q;
      double2 s = make_double2(0.0, 0.0);
      for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
        s.x += red[q][k].x;
        s.y += red[q][k].y;
      }
      if (l < L) alm[(int64_t)m * L + l] = s;
    }
    __syncthreads();
  }
}

// ------------------------------------------------- coefficient operators
// D_inv (cmm_s2/core/spherical_simulations.py:195-198) applied in place;
// entries l < m cleared.
__global__ void dinv_kernel(double2* __restrict__ a, int L) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x, m = blockIdx.y;
  if (l >= L) return;
  const int64_t i = (int64_t)m * L + l;
  if (l < m || l == 0) {
    a[i] = make_double2(0.0, 0.0);
    return;
  }
  const double d = -1.0 / ((double)l * (double)(l + 1));
  a[i] = cmul(a[i], d);
}

// i(L_x, L_y, L_z) of angular_momentum (spherical_harmonic_tools.py:49-62)
// on the m >= 0 half of a real field: up = sqrt(l(l+1)-m(m-1)) a_{l,m-1},
// dn = sqrt(l(l+1)-m(m+1)) a_{l,m+1}, a_{l,-1} = -conj(a_{l,1});
// iLx a = i (up+dn)/2, iLy a = (up-dn)/2, iLz a = i m a.
__device__ __forceinline__ void ladder(const double2* __restrict__ a, int L, int l, int m,
                                       double2* o) {
  const double ll = (double)l * (double)(l + 1);
  double2 am1, ap1;
  if (m == 0) {
    am1 = (l >= 1) ? a[(int64_t)1 * L + l] : make_double2(0.0, 0.0);
    am1 = make_double2(-am1.x, am1.y);  // -conj
  } else {
    am1 = a[(int64_t)(m - 1) * L + l];
  }
  ap1 = (m + 1 <= l) ? a[(int64_t)(m + 1) * L + l] : make_double2(0.0, 0.0);
  const double cu = sqrt(ll - (double)m * (double)(m - 1));
  const double cd = sqrt(ll - (double)m * (double)(m + 1));
  const double2 up = make_double2(cu * am1.x, cu * am1.y);
  const double2 dn = make_double2(cd * ap1.x, cd * ap1.y);
  const double2 sx = make_double2((up.x + dn.x) / 2, (up.y + dn.y) / 2);
  o[0] = make_double2(-sx.y, sx.x);                                   // i * sx
  o[1] = make_double2((up.x - dn.x) / 2, (up.y - dn.y) / 2);
  const double2 am = a[(int64_t)m * L + l];
  o[2] = make_double2(-(double)m * am.y, (double)m * am.x);           // i m a
}

// fields[f] (f = 0..11): 0..2 = u_i = iL_i psi; 3 + 3i + k = iL_k u_i.
__global__ void ladder1_kernel(const double2* __restrict__ psi, int L, double2* __restrict__ fields) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x, m = blockIdx.y;
  if (l >= L) return;
  const int64_t fs = (int64_t)L * L, i = (int64_t)m * L + l;
  if (l < m) {
    for (int f = 0; f < 3; ++f) fields[f * fs + i] = make_double2(0.0, 0.0);
    return;
  }
  double2 o[3];
  ladder(psi, L, l, m, o);
  for (int f = 0; f < 3; ++f) fields[f * fs + i] = o[f];
}

__global__ void ladder2_kernel(double2* __restrict__ fields, int L) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x, m = blockIdx.y;
  if (l >= L) return;
  const int64_t fs = (int64_t)L * L, i = (int64_t)m * L + l;
  for (int u = 0; u < 3; ++u) {
    double2 o[3] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
    if (l >= m) ladder(fields + u * fs, L, l, m, o);
    for (int k = 0; k < 3; ++k) fields[(3 + 3 * u + k) * fs + i] = o[k];
  }
}

// power[l] = sum over all orders -l..l of |a_lm|^2 = |a_l0|^2 + 2 sum_{m>0}
// |a_lm|^2 (real field); one block per degree.  The summand of
// energy_spectrum (cmm_s2/core/spherical_harmonic_tools.py:157-163).
__global__ void power_kernel(const double2* __restrict__ a, int L, double* __restrict__ power) {
  const int l = blockIdx.x;
  double s = 0.0;
  for (int m = threadIdx.x; m <= l; m += blockDim.x) {
    const double2 v = a[(int64_t)m * L + l];
    s += (m == 0 ? 1.0 : 2.0) * (v.x * v.x + v.y * v.y);
  }
  __shared__ double red[8];
  for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    power[l] = t;
  }
}

// fields 0..3 = a, iLx a, iLy a, iLz a (project_onto_S12,
// spherical_harmonic_tools.py:121-123).
__global__ void scalar_fields_kernel(const double2* __restrict__ a, int L, double2* __restrict__ fields) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x, m = blockIdx.y;
  if (l >= L) return;
  const int64_t fs = (int64_t)L * L, i = (int64_t)m * L + l;
  double2 o[3] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
  if (l >= m) ladder(a, L, l, m, o);
  fields[i] = (l >= m) ? a[i] : make_double2(0.0, 0.0);
  for (int k = 0; k < 3; ++k) fields[(1 + k) * fs + i] = o[k];
}

// Scalar jets (4, Nv_u): value, then the tangent gradient
// g x X - ((g x X).X/|X|) X with g = (iLx, iLy, iLz) f (:125-138).
__global__ void scalar_jets_kernel(const double* __restrict__ fld, int L, const double* __restrict__ grid,
                                   double* __restrict__ jets) {
  const int N = 2 * L;
  const int64_t nv = 2 + (int64_t)(L - 1) * N;
  const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const int64_t node = v == 0 ? 0 : (v == nv - 1 ? (int64_t)L * N : N + (v - 1));
  const int64_t fs = (int64_t)(L + 1) * N;
  const double X0 = grid[4 * node], X1 = grid[4 * node + 1], X2 = grid[4 * node + 2];
  const double nX = sqrt(X0 * X0 + X1 * X1 + X2 * X2);
  const double g0 = fld[fs + node], g1 = fld[2 * fs + node], g2 = fld[3 * fs + node];
  const double c0 = g1 * X2 - g2 * X1, c1 = g2 * X0 - g0 * X2, c2 = g0 * X1 - g1 * X0;
  const double sc = (c0 * X0 + c1 * X1 + c2 * X2) / nX;
  jets[v] = fld[node];
  jets[nv + v] = c0 - sc * X0;
  jets[2 * nv + v] = c1 - sc * X1;
  jets[3 * nv + v] = c2 - sc * X2;
}

// ------------------------------------------------------------- inverse
// Legendre synthesis of nf fields: block (m, ring-pair tile); each thread
// one ring pair (t, L-t).  Out: spectra S[f][t][m] (nf, L+1, L+1), m = L
// column zero (written by the caller's memset).
template <int NF>
__global__ void __launch_bounds__(kSynthBlock) synthesis_kernel(const double2* __restrict__ alm, int L,
                                                                const double* __restrict__ ct,
                                                                const double* __restrict__ pmm,
                                                                const double* __restrict__ ra,
                                                                const double* __restrict__ rb,
                                                                double2* __restrict__ S) {
  const int m = blockIdx.x;
  const int t = blockIdx.y * blockDim.x + threadIdx.x;  // 0..L/2
  const int npair = L / 2 + 1;
  const int64_t fs = (int64_t)L * L;
  __shared__ double2 A[kLChunk][NF];
  double2 E[NF], O[NF];
#pragma unroll
  for (int f = 0; f < NF; ++f) E[f] = O[f] = make_double2(0.0, 0.0);
  const bool active = t < npair;
  const double x = active ? ct[t] : 0.0;
  double p0 = active ? pmm[(int64_t)m * (L + 1) + t] : 0.0, p1 = 0.0;
  for (int l0 = m; l0 < L; l0 += kLChunk) {
    __syncthreads();
    for (int e = threadIdx.x; e < kLChunk * NF; e += blockDim.x) {
      const int q = e / NF, f = e % NF, l = l0 + q;
      A[q][f] = (l < L) ? alm[f * fs + (int64_t)m * L + l] : make_double2(0.0, 0.0);
    }
    __syncthreads();
    const int qn = min(kLChunk, L - l0);
    for (int q = 0; q < qn; ++q) {
      const int l = l0 + q;
      double P;
      if (l == m) {
        P = p0;
      } else if (l == m + 1) {
        P = ra[(int64_t)m * L + l] * x * p0;
        p1 = p0;
        p0 = P;
      } else {
        P = ra[(int64_t)m * L + l] * (x * p0 - rb[(int64_t)m * L + l] * p1);
        p1 = p0;
        p0 = P;
      }
      if (((l - m) & 1) == 0) {
#pragma unroll
        for (int f = 0; f < NF; ++f) {
          E[f].x += P * A[q][f].x;
          E[f].y += P * A[q][f].y;
        }
      } else {
#pragma unroll
        for (int f = 0; f < NF; ++f) {
          O[f].x += P * A[q][f].x;
          O[f].y += P * A[q][f].y;
        }
      }
    }
  }
  if (!active) return;
  const int64_t row = L + 1;
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    const int64_t base = (int64_t)f * (L + 1) * row;
    S[base + (int64_t)t * row + m] = make_double2(E[f].x + O[f].x, E[f].y + O[f].y);
    if (L - t != t) S[base + (int64_t)(L - t) * row + m] = make_double2(E[f].x - O[f].x, E[f].y - O[f].y);
  }
}

// ------------------------------------- small band-limits: Pbar tables
// At small L the recurrence kernels above run a few warps per SM (one
// block per m, one thread per ring pair) and are latency-bound, and the
// analysis spends 3 FP64 operations of recurrence per 2 of contraction.
// With tables the Pbar_lm values are computed once per plan (FP64, the same
// recurrence) and both Legendre stages become table contractions with one
// thread per (m, l) (analysis) or per (m, ring pair, field group)
// (synthesis): L^3/2 and L^3/4 doubles, 68 + 34 MB at L = 256, 0.54 + 0.27
// GB at L = 512, 4.3 + 2.2 GB at L = 1024.  By default (cmm_sht_set_tables)
// plans with L <= kTabMaxL use them.
constexpr int kTabMaxL = 512;
constexpr int kTabShared = 1024;   // largest L the analysis kernel's shared arrays hold

// offset of order m in a table with nj entries per (m, l): nj sum_{m'<m} (L - m')
__device__ __host__ __forceinline__ int64_t tab_off(int m, int L, int nj) {
  return (int64_t)nj * ((int64_t)m * L - (int64_t)m * (m - 1) / 2);
}

// One thread per (m, ring j): Pbar_{l,m}(theta_j), l = m..L-1.  lmajor:
// layout [m][l-m][j] (synthesis) else [m][j][l-m] (analysis).
__global__ void build_pbar_kernel(int L, int nj, const double* __restrict__ ct, const double* __restrict__ pmm,
                                  int pmm_stride, const double* __restrict__ ra, const double* __restrict__ rb,
                                  bool lmajor, double* __restrict__ tab) {
  const int m = blockIdx.y, j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nj) return;
  const double x = ct[j];
  double p0 = pmm[(int64_t)m * pmm_stride + j], p1 = 0.0;
  double* base = tab + tab_off(m, L, nj);
  const int nl = L - m;
  for (int l = m; l < L; ++l) {
    double P;
    if (l == m) {
      P = p0;
    } else if (l == m + 1) {
      P = ra[(int64_t)m * L + l] * x * p0;
      p1 = p0;
      p0 = P;
    } else {
      P = ra[(int64_t)m * L + l] * (x * p0 - rb[(int64_t)m * L + l] * p1);
      p1 = p0;
      p0 = P;
    }
    const int i = l - m;
    base[lmajor ? (int64_t)i * nj + j : (int64_t)j * nl + i] = P;
  }
}

// Analysis from the table: block (m, tile of 64 degrees), thread l; the
// weighted even/odd ring spectra of order m staged in shared memory.
constexpr int kTabBlock = 64;
__global__ void __launch_bounds__(kTabBlock) analysis_tab_kernel(const double2* __restrict__ fine, int L,
                                                                 const double* __restrict__ w,
                                                                 const double* __restrict__ tab,
                                                                 double2* __restrict__ alm) {
  __shared__ double2 E[kTabShared + 1], O[kTabShared + 1];
  const int m = blockIdx.x, l = m + blockIdx.y * kTabBlock + threadIdx.x;
  if (m + (int)blockIdx.y * kTabBlock >= L) return;   // the whole tile is past l = L-1
  const int npair = L + 1;
  for (int j = threadIdx.x; j < npair; j += blockDim.x) {
    const double2 a = fine[(int64_t)m * 4 * L + j];
    double2 e, o;
    if (j < L) {
      const double2 b = fine[(int64_t)m * 4 * L + 2 * L - j];
      e = make_double2(a.x + b.x, a.y + b.y);
      o = make_double2(a.x - b.x, a.y - b.y);
    } else {
      e = a;
      o = make_double2(0.0, 0.0);
    }
    E[j] = cmul(e, w[j]);
    O[j] = cmul(o, w[j]);
  }
  __syncthreads();
  if (l >= L) return;
  const int nl = L - m, i = l - m;
  const double* P = tab + tab_off(m, L, npair) + i;
  const double2* V = (i & 1) == 0 ? E : O;
  double2 acc = make_double2(0.0, 0.0);
  for (int j = 0; j < npair; ++j) {
    const double pj = __ldg(P + (int64_t)j * nl);
    acc.x += pj * V[j].x;
    acc.y += pj * V[j].y;
  }
  alm[(int64_t)m * L + l] = acc;
}

// Synthesis from the table: block (m, tile of ring pairs, group of G
// fields); each thread one ring pair (t, L-t) and G fields.
template <int G>
__global__ void __launch_bounds__(kTabBlock) synthesis_tab_kernel(const double2* __restrict__ alm, int L,
                                                                  const double* __restrict__ tab,
                                                                  double2* __restrict__ S) {
  const int m = blockIdx.x, t = blockIdx.y * blockDim.x + threadIdx.x, f0 = blockIdx.z * G;
  const int npair = L / 2 + 1;
  const int64_t fs = (int64_t)L * L;
  __shared__ double2 A[kLChunk][G];
  double2 E[G], O[G];
#pragma unroll
  for (int f = 0; f < G; ++f) E[f] = O[f] = make_double2(0.0, 0.0);
  const bool active = t < npair;
  const double* P = tab + tab_off(m, L, npair) + (active ? t : 0);
  for (int l0 = m; l0 < L; l0 += kLChunk) {
    __syncthreads();
    for (int e = threadIdx.x; e < kLChunk * G; e += blockDim.x) {
      const int q = e / G, f = e % G, l = l0 + q;
      A[q][f] = (l < L) ? alm[(f0 + f) * fs + (int64_t)m * L + l] : make_double2(0.0, 0.0);
    }
    __syncthreads();
    const int qn = min(kLChunk, L - l0);
    for (int q = 0; q < qn; ++q) {
      const int l = l0 + q;
      const double pv = active ? __ldg(P + (int64_t)(l - m) * npair) : 0.0;
      if (((l - m) & 1) == 0) {
#pragma unroll
        for (int f = 0; f < G; ++f) {
          E[f].x += pv * A[q][f].x;
          E[f].y += pv * A[q][f].y;
        }
      } else {
#pragma unroll
        for (int f = 0; f < G; ++f) {
          O[f].x += pv * A[q][f].x;
          O[f].y += pv * A[q][f].y;
        }
      }
    }
  }
  if (!active) return;
  const int64_t row = L + 1;
#pragma unroll
  for (int f = 0; f < G; ++f) {
    const int64_t base = (int64_t)(f0 + f) * (L + 1) * row;
    S[base + (int64_t)t * row + m] = make_double2(E[f].x + O[f].x, E[f].y + O[f].y);
    if (L - t != t) S[base + (int64_t)(L - t) * row + m] = make_double2(E[f].x - O[f].x, E[f].y - O[f].y);
  }
}

// Velocity jets (project_stream, spherical_harmonic_tools.py:81-101) from
// the 12 synthesised fields on the grid: vals[i][0] = u_i and, with
// g = (iLx, iLy, iLz) u_i, vals[c][1+i] = (g x X - ((g x X).X/|X|) X)_c;
// poles from sample 0 of the first and last rings.
// jets_f (nullable): the same values as floats (exact for R = float).
template <typename R>
__global__ void jets_kernel(const R* __restrict__ fld, int L, const double* __restrict__ grid,
                            double* __restrict__ jets, float* __restrict__ jets_f) {
  const int N = 2 * L;
  const int64_t nv = 2 + (int64_t)(L - 1) * N;
  const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (v >= nv) return;
  int64_t node;  // ring * N + p
  if (v == 0)
    node = 0;
  else if (v == nv - 1)
    node = (int64_t)L * N;
  else
    node = N + (v - 1);
  const int64_t fs = (int64_t)(L + 1) * N;
  // arithmetic in the samples' precision (FP32 in the mixed form)
  const R X0 = (R)grid[4 * node], X1 = (R)grid[4 * node + 1], X2 = (R)grid[4 * node + 2];
  const R nX = sqrt(X0 * X0 + X1 * X1 + X2 * X2);
  for (int i = 0; i < 3; ++i) {
    const R g0 = fld[(3 + 3 * i) * fs + node], g1 = fld[(4 + 3 * i) * fs + node],
            g2 = fld[(5 + 3 * i) * fs + node];
    const R c0 = g1 * X2 - g2 * X1, c1 = g2 * X0 - g0 * X2, c2 = g0 * X1 - g1 * X0;
    const R sc = (c0 * X0 + c1 * X1 + c2 * X2) / nX;
    const R val[4] = {fld[i * fs + node], c0 - sc * X0, c1 - sc * X1, c2 - sc * X2};
    const int64_t slot[4] = {i * 4, 0 * 4 + 1 + i, 1 * 4 + 1 + i, 2 * 4 + 1 + i};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      jets[slot[k] * nv + v] = (double)val[k];
      if (jets_f) jets_f[slot[k] * nv + v] = (float)val[k];
    }
  }
}

// ------------------------------------------------------------ adjoint
// Transposes of the stages of sht_velocity (exact transposes of the
// linear maps, complex arrays taken as pairs of reals).

// sum over rings: out[m][l] = sum_{j=0..nr} w_j c_m Pbar_lm(theta_j) F[j][m],
// rings j and nr-j paired (Pbar(pi - theta) = (-1)^(l+m) Pbar(theta)),
// F row stride `row`, c_0 = 1 and c_m = cm (m > 0); w == NULL: unit weights.
// blockIdx.y selects one of several fields (F + y fstride_in, out + y fstride_out);
// R ring pairs per thread (256 R >= nr/2 + 1).
template <int R, int C = 16>
__global__ void __launch_bounds__(256) legendre_sum_kernel(const double2* __restrict__ F, int64_t row, int L,
                                                           int nr, const double* __restrict__ w, double cm,
                                                           const double* __restrict__ ct,
                                                           const double* __restrict__ pmm, int pstride,
                                                           const double* __restrict__ ra,
                                                           const double* __restrict__ rb,
                                                           double2* __restrict__ out, int64_t fs_in,
                                                           int64_t fs_out) {
  const int m = blockIdx.x;
  F += blockIdx.y * fs_in;
  out += blockIdx.y * fs_out;
  const int npair = nr / 2 + 1;
  const double sc = m == 0 ? 1.0 : cm;
  double2 E[R], O[R];
  double x[R], p0[R], p1[R];
  int nrr = 0;
  for (int r = 0; r < R; ++r) {
    const int j = threadIdx.x + r * blockDim.x;
    if (j < npair) {
      const double2 a = F[(int64_t)j * row + m];
      double2 e, o;
      if (j < nr - j) {
        const double2 b = F[(int64_t)(nr - j) * row + m];
        e = make_double2(a.x + b.x, a.y + b.y);
        o = make_double2(a.x - b.x, a.y - b.y);
      } else {
        e = a;
        o = make_double2(0.0, 0.0);
      }
      const double wj = (w ? w[j] : 1.0) * sc;
      E[r] = cmul(e, wj);
      O[r] = cmul(o, wj);
      x[r] = ct[j];
      p0[r] = pmm[(int64_t)m * pstride + j];
      p1[r] = 0.0;
      nrr = r + 1;
    } else {
      E[r] = O[r] = make_double2(0.0, 0.0);
      x[r] = p0[r] = p1[r] = 0.0;
    }
  }
  __shared__ double2 red[C][8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int l0 = m; l0 < L; l0 += C) {
    double2 acc[C];
#pragma unroll
    for (int q = 0; q < C; ++q) acc[q] = make_double2(0.0, 0.0);
#pragma unroll
    for (int q = 0; q < C; ++q) {
      const int l = l0 + q;
      if (l < L) {
        const bool even = ((l - m) & 1) == 0;
        double a = 0.0, b = 0.0;
        if (l > m) {
          a = ra[(int64_t)m * L + l];
          b = rb[(int64_t)m * L + l];
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
          if (r < nrr) {
            double P;
            if (l == m) {
              P = p0[r];
            } else if (l == m + 1) {
              P = a * x[r] * p0[r];
              p1[r] = p0[r];
              p0[r] = P;
            } else {
              P = a * (x[r] * p0[r] - b * p1[r]);
              p1[r] = p0[r];
              p0[r] = P;
            }
            const double2 v = even ? E[r] : O[r];
            acc[q].x += P * v.x;
            acc[q].y += P * v.y;
          }
        }
      }
    }
#pragma unroll
    for (int q = 0; q < C; ++q) {
      double vx = acc[q].x, vy = acc[q].y;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        vx += __shfl_down_sync(0xffffffffu, vx, off);
        vy += __shfl_down_sync(0xffffffffu, vy, off);
      }
      if (lane == 0) red[q][warp] = make_double2(vx, vy);
    }
    __syncthreads();
    if (threadIdx.x < C) {
      const int q = threadIdx.x, l = l0 + q;
      double2 s = make_double2(0.0, 0.0);
      for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
        s.x += red[q][k].x;
        s.y += red[q][k].y;
      }
      if (l < L) out[(int64_t)m * L + l] = s;
    }
    __syncthreads();
  }
}

// legendre_sum_kernel on the synthesis Pbar table (unit weights, the L+1
// MWSS rings, pairs (t, L-t)) for NF fields: block (m, tile of 64 degrees,
// group of G fields), one thread per degree l; the group's weighted even/odd
// ring values of order m staged in shared memory, the thread's table row
// streamed over the ring pairs.
template <int G>
__global__ void __launch_bounds__(kTabBlock) legendre_sum_tab_kernel(const double2* __restrict__ F,
                                                                     int64_t row, int L, double cm,
                                                                     const double* __restrict__ tab,
                                                                     double2* __restrict__ out, int64_t fs_in,
                                                                     int64_t fs_out) {
  constexpr int kMaxPair = kTabShared / 2 + 1;
  __shared__ double2 E[G][kMaxPair], O[G][kMaxPair];
  const int m = blockIdx.x, l = m + blockIdx.y * kTabBlock + threadIdx.x, f0 = blockIdx.z * G;
  if (m + (int)blockIdx.y * kTabBlock >= L) return;   // the whole tile is past l = L-1
  const int nr = L, npair = nr / 2 + 1;
  const double sc = m == 0 ? 1.0 : cm;
  for (int e = threadIdx.x; e < G * npair; e += blockDim.x) {
    const int f = e / npair, j = e % npair;
    const double2* Ff = F + (int64_t)(f0 + f) * fs_in;
    const double2 a = Ff[(int64_t)j * row + m];
    double2 ev, od;
    if (j < nr - j) {
      const double2 b = Ff[(int64_t)(nr - j) * row + m];
      ev = make_double2(a.x + b.x, a.y + b.y);
      od = make_double2(a.x - b.x, a.y - b.y);
    } else {
      ev = a;
      od = make_double2(0.0, 0.0);
    }
    E[f][j] = cmul(ev, sc);
    O[f][j] = cmul(od, sc);
  }
  __syncthreads();
  if (l >= L) return;
  const int i = l - m;
  const double* P = tab + tab_off(m, L, npair) + (int64_t)i * npair;
  const bool even = (i & 1) == 0;
  double2 acc[G];
#pragma unroll
  for (int f = 0; f < G; ++f) acc[f] = make_double2(0.0, 0.0);
  for (int j = 0; j < npair; ++j) {
    const double pj = __ldg(P + j);
#pragma unroll
    for (int f = 0; f < G; ++f) {
      const double2 v = even ? E[f][j] : O[f][j];
      acc[f].x += pj * v.x;
      acc[f].y += pj * v.y;
    }
  }
#pragma unroll
  for (int f = 0; f < G; ++f) out[(int64_t)(f0 + f) * fs_out + (int64_t)m * L + l] = acc[f];
}

// ring synthesis with weights: out[j][m] = w_j sum_l Pbar_lm(theta_j)
// a[m][l] for rings j = 0..nr (pairs j, nr-j), rows of length `row`.
__global__ void __launch_bounds__(kSynthBlock) ring_synthesis_kernel(const double2* __restrict__ alm, int L,
                                                                     int nr, const double* __restrict__ w,
                                                                     const double* __restrict__ ct,
                                                                     const double* __restrict__ pmm,
                                                                     int pstride,
                                                                     const double* __restrict__ ra,
                                                                     const double* __restrict__ rb,
                                                                     double2* __restrict__ out, int64_t row) {
  const int m = blockIdx.x;
  const int t = blockIdx.y * blockDim.x + threadIdx.x;
  const int npair = nr / 2 + 1;
  __shared__ double2 A[kLChunk];
  double2 E = make_double2(0.0, 0.0), O = make_double2(0.0, 0.0);
  const bool active = t < npair;
  const double x = active ? ct[t] : 0.0;
  double p0 = active ? pmm[(int64_t)m * pstride + t] : 0.0, p1 = 0.0;
  for (int l0 = m; l0 < L; l0 += kLChunk) {
    __syncthreads();
    for (int e = threadIdx.x; e < kLChunk; e += blockDim.x) {
      const int l = l0 + e;
      A[e] = (l < L) ? alm[(int64_t)m * L + l] : make_double2(0.0, 0.0);
    }
    __syncthreads();
    const int qn = min(kLChunk, L - l0);
    for (int q = 0; q < qn; ++q) {
      const int l = l0 + q;
      double P;
      if (l == m) {
        P = p0;
      } else if (l == m + 1) {
        P = ra[(int64_t)m * L + l] * x * p0;
        p1 = p0;
        p0 = P;
      } else {
        P = ra[(int64_t)m * L + l] * (x * p0 - rb[(int64_t)m * L + l] * p1);
        p1 = p0;
        p0 = P;
      }
      if (((l - m) & 1) == 0) {
        E.x += P * A[q].x;
        E.y += P * A[q].y;
      } else {
        O.x += P * A[q].x;
        O.y += P * A[q].y;
      }
    }
  }
  if (!active) return;
  const double wt = w ? w[t] : 1.0;
  out[(int64_t)t * row + m] = make_double2(wt * (E.x + O.x), wt * (E.y + O.y));
  if (nr - t != t) out[(int64_t)(nr - t) * row + m] = make_double2(wt * (E.x - O.x), wt * (E.y - O.y));
}

// jets transpose: jet cotangents (3,4,Nv_u) -> field cotangents (12, L+1, 2L)
// at the vertices' grid nodes (other pole samples stay 0): values, and
// gbar = X x hbar for the tangent-gradient slots (the forward's projection
// term (g x X).X vanishes identically).
__global__ void jets_bwd_kernel(const double* __restrict__ gj, int L, const double* __restrict__ grid,
                                double* __restrict__ gf) {
  const int N = 2 * L;
  const int64_t nv = 2 + (int64_t)(L - 1) * N;
  const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const int64_t node = v == 0 ? 0 : (v == nv - 1 ? (int64_t)L * N : N + (v - 1));
  const int64_t fs = (int64_t)(L + 1) * N;
  const double X0 = grid[4 * node], X1 = grid[4 * node + 1], X2 = grid[4 * node + 2];
  for (int i = 0; i < 3; ++i) {
    gf[i * fs + node] = gj[(int64_t)(i * 4) * nv + v];
    const double h0 = gj[(int64_t)(0 * 4 + 1 + i) * nv + v], h1 = gj[(int64_t)(1 * 4 + 1 + i) * nv + v],
                 h2 = gj[(int64_t)(2 * 4 + 1 + i) * nv + v];
    gf[(3 + 3 * i) * fs + node] = X1 * h2 - X2 * h1;
    gf[(4 + 3 * i) * fs + node] = X2 * h0 - X0 * h2;
    gf[(5 + 3 * i) * fs + node] = X0 * h1 - X1 * h0;
  }
}

// Transpose of `ladder` (gather form): cotangents ob[k] (k = x, y, z) of
// the three outputs at every (m', l) -> cotangent of the input at (m, l).
__device__ __forceinline__ double2 ladder_t(const double2* __restrict__ ox, const double2* __restrict__ oy,
                                            const double2* __restrict__ oz, int L, int l, int m) {
  const double ll = (double)l * (double)(l + 1);
  auto idx = [&](int mm) { return (int64_t)mm * L + l; };
  // up/dn cotangents of the output at m': up = (-i ox + oy)/2, dn = (-i ox - oy)/2
  auto upb = [&](int mm) {
    const double2 a = ox[idx(mm)], b = oy[idx(mm)];
    return make_double2((a.y + b.x) / 2, (-a.x + b.y) / 2);
  };
  auto dnb = [&](int mm) {
    const double2 a = ox[idx(mm)], b = oy[idx(mm)];
    return make_double2((a.y - b.x) / 2, (-a.x - b.y) / 2);
  };
  double2 r = make_double2(0.0, 0.0);
  // output m+1 reads a[m] as am1 (cu(l, m+1))
  if (m + 1 <= l) {
    const double cu = sqrt(ll - (double)(m + 1) * (double)m);
    const double2 u = upb(m + 1);
    r.x += cu * u.x;
    r.y += cu * u.y;
  }
  // output m-1 reads a[m] as ap1 (cd(l, m-1))
  if (m >= 1) {
    const double cd = sqrt(ll - (double)(m - 1) * (double)m);
    const double2 d = dnb(m - 1);
    r.x += cd * d.x;
    r.y += cd * d.y;
  }
  // output m = 0 reads a[1] as am1 = -conj(a[1]) (cu(l, 0))
  if (m == 1) {
    const double cu0 = sqrt(ll);
    const double2 u = upb(0);
    r.x += -cu0 * u.x;
    r.y += cu0 * u.y;
  }
  // o_z = i m a
  const double2 z = oz[idx(m)];
  r.x += (double)m * z.y;
  r.y += -(double)m * z.x;
  return r;
}

// fields cotangents: fb[u] += ladder^T(fb[3+3u .. 5+3u]) (u = 0..2), then
// psib = ladder^T(fb[0..2]); entries l < m are zero.
__global__ void ladder2_bwd_kernel(double2* __restrict__ fb, int L) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x, m = blockIdx.y;
  if (l >= L || l < m) return;
  const int64_t fs = (int64_t)L * L, i = (int64_t)m * L + l;
  for (int u = 0; u < 3; ++u) {
    const double2 r = ladder_t(fb + (3 + 3 * u) * fs, fb + (4 + 3 * u) * fs, fb + (5 + 3 * u) * fs, L, l, m);
    fb[u * fs + i].x += r.x;
    fb[u * fs + i].y += r.y;
  }
}

__global__ void ladder1_bwd_kernel(const double2* __restrict__ fb, int L, double2* __restrict__ psib) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x, m = blockIdx.y;
  if (l >= L) return;
  const int64_t fs = (int64_t)L * L, i = (int64_t)m * L + l;
  psib[i] = (l < m) ? make_double2(0.0, 0.0) : ladder_t(fb, fb + fs, fb + 2 * fs, L, l, m);
}

// pad transpose: Hb (4L, L) -> Ghb (2L, L).
__global__ void pad_bwd_kernel(const double2* __restrict__ Hb, int L, double2* __restrict__ Gb) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y;  // 0..2L-1
  if (m >= L || k >= 2 * L) return;
  const double s = 1.0 / (2 * L);
  double2 v;
  if (k < L) {
    v = Hb[(int64_t)k * L + m];
  } else if (k == L) {
    const double2 a = Hb[(int64_t)L * L + m], b = Hb[(int64_t)3 * L * L + m];
    v = make_double2((a.x + b.x) / 2, (a.y + b.y) / 2);
  } else {
    v = Hb[(int64_t)(k + 2 * L) * L + m];
  }
  Gb[(int64_t)k * L + m] = cmul(v, s);
}

// torus transpose + C2R preparation: Gb (2L, L) -> X (L+1, L+1) with
// specb[t][m] = (pi/L) (Gb[t][m] + [0<t<L] (-1)^m Gb[2L-t][m]), scaled by
// 1/2 for 1 <= m < L (C2R doubles those), m = L zero.
__global__ void torus_bwd_kernel(const double2* __restrict__ Gb, int L, double2* __restrict__ X) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  const int t = blockIdx.y;  // 0..L
  if (m > L || t > L) return;
  double2 v = make_double2(0.0, 0.0);
  if (m < L) {
    v = Gb[(int64_t)t * L + m];
    if (t > 0 && t < L) {
      double2 b = Gb[(int64_t)(2 * L - t) * L + m];
      if (m & 1) b = make_double2(-b.x, -b.y);
      v.x += b.x;
      v.y += b.y;
    }
    v = cmul(v, M_PI / L * (m == 0 ? 1.0 : 0.5));
  }
  X[(int64_t)t * (L + 1) + m] = v;
}

int cufft_fail(cufftResult r, const char* what) {
  set_last_error(std::string(what) + ": cuFFT error " + std::to_string((int)r));
  return CMM_ERR_CUDA;
}

int check_launch(const char* what) {
  note_launch();
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? CMM_OK : cuda_fail(e, what);
}

}  // namespace
}  // namespace cmm

struct cmm_sht {
  int L = 0;
  int precision = CMM_SHT_FP64;
  cufftHandle ring_fwd = 0, torus_fwd = 0, pad_inv = 0, ring_inv = 0;
  bool have_plans[4] = {false, false, false, false};
  // FP64 forward on order-major rows (torus_t_kernel / pad_t_kernel)
  cufftHandle torus_fwd_t = 0, pad_inv_t = 0;
  bool have_tplans[2] = {false, false};
  cmm::DeviceBuffer ct_rings, ct_fine, w_fine, pmm_rings, pmm_fine, ra, rb;
  // Pbar tables of the FP64 stages (analysis a, synthesis s); plans of one
  // band-limit may hold the same tables (cmm_sht_share_tables)
  struct PbarTables {
    cmm::DeviceBuffer a, s;
  };
  std::shared_ptr<PbarTables> tab;
  int tab_mode = 0;                 // cmm_sht_set_tables: 0 auto, 1 always, -1 never
  cmm::DeviceBuffer spec, torus, pad, alm, fields, synth, samples, status;
  cmm::TcPlan* tc = nullptr;
  int tc_schedule = 1;   // split-BF16 synthesis schedule (cmm_sht_set_schedule)
  // split-BF16 form: FP32 ring FFTs and buffers, made with the tc plan
  cufftHandle f_ring_fwd = 0, f_torus_fwd = 0, f_pad_inv = 0, f_ring_inv = 0;
  bool have_fplans[4] = {false, false, false, false};
  cmm::DeviceBuffer f_in, f_spec, f_torus, f_pad, f_synth, f_samples;
  // the velocity jets of the split form also as the FP32 values they are
  // computed in (12 x Nv_u floats), which the FP32 velocity assembly reads
  cmm::DeviceBuffer f_jets;
  // adjoint: D2Z over the 12 fields' rings, C2R over one field's rings
  cufftHandle b_ring_fwd12 = 0, b_ring_inv1 = 0;
  bool have_bplans = false;
  // batch membership (cmm_sht_batch_create): the batch and this plan's slot
  cmm_sht_batch* batch = nullptr;
  int slot = -1;
  ~cmm_sht();
};

// Up to 8 split-BF16 plans of one band-limit whose forward analyses run as
// one tensor-core launch: each member writes its data tiles into column
// pair `slot` of the shared 16-column tiles (sht_velocity_pre, inside
// cmm_bve_step_pre or cmm_sht_batch_forward), then one contraction streams
// every Pbar tile once for all members (cmm_sht_batch_analysis).
struct cmm_sht_batch {
  int L = 0, n = 0;
  cmm_sht* plans[8] = {};
  cmm::DeviceBuffer xtab;
};

cmm_sht::~cmm_sht() {
  {
    if (have_plans[0]) cufftDestroy(ring_fwd);
    if (have_plans[1]) cufftDestroy(torus_fwd);
    if (have_plans[2]) cufftDestroy(pad_inv);
    if (have_plans[3]) cufftDestroy(ring_inv);
    if (have_tplans[0]) cufftDestroy(torus_fwd_t);
    if (have_tplans[1]) cufftDestroy(pad_inv_t);
    if (have_fplans[0]) cufftDestroy(f_ring_fwd);
    if (have_fplans[1]) cufftDestroy(f_torus_fwd);
    if (have_fplans[2]) cufftDestroy(f_pad_inv);
    if (have_fplans[3]) cufftDestroy(f_ring_inv);
    if (have_bplans) {
      cufftDestroy(b_ring_fwd12);
      cufftDestroy(b_ring_inv1);
    }
    if (tc) cmm::tc_plan_destroy(tc);
    // a plan destroyed before its batch leaves an empty slot, which the
    // batch's analysis reports as an error
    if (batch) batch->plans[slot] = nullptr;
  }
}

namespace cmm {

// Sectoral start values Pbar_mm(theta_j) (L, nring) and the recurrence
// coefficients a_lm = sqrt((4l^2-1)/(l^2-m^2)), b_lm = sqrt(((l-1)^2-m^2)/
// (4(l-1)^2-1)) (m-major (L, L)); a_{m+1,m} = sqrt(2m+3).
static void legendre_tables(int L, const std::vector<double>& theta, std::vector<double>& pmm,
                            std::vector<double>& ct) {
  const int n = (int)theta.size();
  pmm.assign((size_t)L * n, 0.0);
  ct.resize(n);
  for (int j = 0; j < n; ++j) {
    const double x = std::cos(theta[j]), s = std::sin(theta[j]);
    ct[j] = x;
    double p = std::sqrt(1.0 / (4.0 * M_PI));
    for (int m = 0; m < L; ++m) {
      if (m > 0) p = -p * std::sqrt((2.0 * m + 1.0) / (2.0 * m)) * s;
      pmm[(size_t)m * n + j] = p;
    }
  }
}

int sht_create(int L, cmm_sht** out) {
  if (L < 2 || L > 4096) {
    set_last_error("cmm_sht_create: L must be in [2, 4096]");
    return CMM_ERR_ARG;
  }
  cmm_sht* p = new (std::nothrow) cmm_sht();
  if (!p) {
    set_last_error("cmm_sht_create: out of host memory");
    return CMM_ERR_NOMEM;
  }
  p->L = L;
  std::vector<double> th(L + 1), thf(2 * L + 1), w(2 * L + 1);
  for (int t = 0; t <= L; ++t) th[t] = M_PI * t / L;
  for (int j = 0; j <= 2 * L; ++j) thf[j] = M_PI * j / (2 * L);
  // Clenshaw-Curtis weights on 2L+1 points (M = 2L even)
  const int M = 2 * L;
  for (int j = 0; j <= M; ++j) {
    double s = 1.0;
    for (int k = 1; k <= M / 2; ++k) {
      const double b = (k == M / 2) ? 1.0 : 2.0;
      s -= b / (4.0 * k * k - 1.0) * std::cos(2.0 * M_PI * j * k / M);
    }
    w[j] = ((j == 0 || j == M) ? 1.0 : 2.0) / M * s;
  }
  std::vector<double> pmm_r, ct_r, pmm_f, ct_f, ra((size_t)L * L, 0.0), rb((size_t)L * L, 0.0);
  legendre_tables(L, th, pmm_r, ct_r);
  legendre_tables(L, thf, pmm_f, ct_f);
  for (int m = 0; m < L; ++m)
    for (int l = m + 1; l < L; ++l) {
      const double ld = l, md = m;
      if (l == m + 1) {
        ra[(size_t)m * L + l] = std::sqrt(2.0 * md + 3.0);
      } else {
        ra[(size_t)m * L + l] = std::sqrt((4.0 * ld * ld - 1.0) / (ld * ld - md * md));
        rb[(size_t)m * L + l] = std::sqrt(((ld - 1) * (ld - 1) - md * md) / (4.0 * (ld - 1) * (ld - 1) - 1.0));
      }
    }
  int rc;
  auto fail = [&](int r) {
    delete p;
    return r;
  };
  // synthesis uses ring pairs t = 0..L/2 only
  if ((rc = p->ct_rings.upload(ct_r.data(), ct_r.size() * 8))) return fail(rc);
  if ((rc = p->ct_fine.upload(ct_f.data(), ct_f.size() * 8))) return fail(rc);
  if ((rc = p->w_fine.upload(w.data(), w.size() * 8))) return fail(rc);
  if ((rc = p->pmm_rings.upload(pmm_r.data(), pmm_r.size() * 8))) return fail(rc);
  if ((rc = p->pmm_fine.upload(pmm_f.data(), pmm_f.size() * 8))) return fail(rc);
  if ((rc = p->ra.upload(ra.data(), ra.size() * 8))) return fail(rc);
  if ((rc = p->rb.upload(rb.data(), rb.size() * 8))) return fail(rc);
  const size_t c16 = sizeof(double2);
  if ((rc = p->spec.alloc((size_t)(L + 1) * (L + 1) * c16))) return fail(rc);
  if ((rc = p->torus.alloc((size_t)2 * L * L * c16))) return fail(rc);
  if ((rc = p->pad.alloc((size_t)4 * L * L * c16))) return fail(rc);
  if ((rc = p->alm.alloc((size_t)L * L * c16))) return fail(rc);
  if ((rc = p->fields.alloc((size_t)kFields * L * L * c16))) return fail(rc);
  {
    const int zero = 0;
    if ((rc = p->status.upload(&zero, sizeof(int)))) return fail(rc);
  }
  cufftResult r;
  int n2[1] = {2 * L}, n4[1] = {4 * L};
  // rings: (L+1) real rows of 2L -> (L+1) x (L+1) complex
  int inemb[1] = {2 * L}, onemb[1] = {L + 1};
  r = cufftPlanMany(&p->ring_fwd, 1, n2, inemb, 1, 2 * L, onemb, 1, L + 1, CUFFT_D2Z, L + 1);
  if (r != CUFFT_SUCCESS) return fail(cufft_fail(r, "cufftPlanMany(ring_fwd)"));
  p->have_plans[0] = true;
  // torus: L columns of 2L with stride L
  int tn[1] = {2 * L};
  r = cufftPlanMany(&p->torus_fwd, 1, n2, tn, L, 1, tn, L, 1, CUFFT_Z2Z, L);
  if (r != CUFFT_SUCCESS) return fail(cufft_fail(r, "cufftPlanMany(torus_fwd)"));
  p->have_plans[1] = true;
  int pn[1] = {4 * L};
  r = cufftPlanMany(&p->pad_inv, 1, n4, pn, L, 1, pn, L, 1, CUFFT_Z2Z, L);
  if (r != CUFFT_SUCCESS) return fail(cufft_fail(r, "cufftPlanMany(pad_inv)"));
  p->have_plans[2] = true;
  // inverse rings: kFields*(L+1) rows of L+1 complex -> 2L real
  int cin[1] = {L + 1}, rout[1] = {2 * L};
  r = cufftPlanMany(&p->ring_inv, 1, n2, cin, 1, L + 1, rout, 1, 2 * L, CUFFT_Z2D, kFields * (L + 1));
  if (r != CUFFT_SUCCESS) return fail(cufft_fail(r, "cufftPlanMany(ring_inv)"));
  p->have_plans[3] = true;
  r = cufftPlanMany(&p->torus_fwd_t, 1, n2, tn, 1, 2 * L, tn, 1, 2 * L, CUFFT_Z2Z, L);
  if (r != CUFFT_SUCCESS) return fail(cufft_fail(r, "cufftPlanMany(torus_fwd_t)"));
  p->have_tplans[0] = true;
  r = cufftPlanMany(&p->pad_inv_t, 1, n4, pn, 1, 4 * L, pn, 1, 4 * L, CUFFT_Z2Z, L);
  if (r != CUFFT_SUCCESS) return fail(cufft_fail(r, "cufftPlanMany(pad_inv_t)"));
  p->have_tplans[1] = true;
  *out = p;
  return CMM_OK;
}

static int set_streams(cmm_sht* p, cudaStream_t s) {
  cufftHandle h[8] = {p->ring_fwd, p->torus_fwd, p->pad_inv, p->ring_inv,
                      p->f_ring_fwd, p->f_torus_fwd, p->f_pad_inv, p->f_ring_inv};
  for (int k = 0; k < 8; ++k) {
    if (k >= 4 && !p->have_fplans[k - 4]) continue;
    cufftResult r = cufftSetStream(h[k], s);
    if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftSetStream");
  }
  cufftHandle ht[2] = {p->torus_fwd_t, p->pad_inv_t};
  for (int k = 0; k < 2; ++k) {
    if (!p->have_tplans[k]) continue;
    cufftResult r = cufftSetStream(ht[k], s);
    if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftSetStream");
  }
  return CMM_OK;
}

// Pbar tables of the FP64 Legendre stages at L <= kTabMaxL, built at their
// first use on `s` (a call inside a stream capture keeps the recurrence
// kernels, since a capture cannot allocate); released by cmm_sht_trim.
static int ensure_tables(cmm_sht* p, cudaStream_t s, bool* ok) {
  *ok = false;
  const int L = p->L;
  if (p->tab_mode < 0 || (p->tab_mode == 0 && L > kTabMaxL) || L > kTabShared) return CMM_OK;
  if (p->tab) {
    *ok = true;
    return CMM_OK;
  }
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) {
    cudaGetLastError();
    return CMM_OK;
  }
  if (cs != cudaStreamCaptureStatusNone) return CMM_OK;
  const int64_t tri = (int64_t)L * (L + 1) / 2;
  const int na = L + 1, ns = L / 2 + 1;
  int rc;
  auto tab = std::make_shared<cmm_sht::PbarTables>();
  if ((rc = tab->a.alloc((size_t)tri * na * 8)) || (rc = tab->s.alloc((size_t)tri * ns * 8))) return rc;
  build_pbar_kernel<<<dim3((na + 127) / 128, L), 128, 0, s>>>(L, na, (const double*)p->ct_fine.p,
                                                              (const double*)p->pmm_fine.p, 2 * L + 1,
                                                              (const double*)p->ra.p, (const double*)p->rb.p,
                                                              false, (double*)tab->a.p);
  if ((rc = check_launch("build_pbar_kernel"))) return rc;
  build_pbar_kernel<<<dim3((ns + 127) / 128, L), 128, 0, s>>>(L, ns, (const double*)p->ct_rings.p,
                                                              (const double*)p->pmm_rings.p, L + 1,
                                                              (const double*)p->ra.p, (const double*)p->rb.p,
                                                              true, (double*)tab->s.p);
  if ((rc = check_launch("build_pbar_kernel"))) return rc;
  // published only once built: a later call of this plan on another
  // stream, unordered with s, must not read a partly written table
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "build_pbar_kernel");
  p->tab = std::move(tab);
  *ok = true;
  return CMM_OK;
}

// Scratch of the FP64 inverse (spectra and samples of 12 fields, about
// 400 MB at L = 1024), allocated at its first use and released by
// cmm_sht_trim.
static int ensure_fp64_inverse(cmm_sht* p) {
  const int L = p->L;
  int rc;
  if (!p->synth.p && (rc = p->synth.alloc((size_t)kFields * (L + 1) * (L + 1) * sizeof(double2)))) return rc;
  if (!p->samples.p && (rc = p->samples.alloc((size_t)kFields * (L + 1) * 2 * L * 8))) return rc;
  return CMM_OK;
}

// FP32 FFT plans and buffers of the split-BF16 form (same shapes as the
// FP64 plans of sht_create).
static int make_float_plans(cmm_sht* p) {
  const int L = p->L;
  int rc;
  if ((rc = p->f_in.alloc((size_t)(L + 1) * 2 * L * sizeof(float))) ||
      (rc = p->f_spec.alloc((size_t)(L + 1) * (L + 1) * sizeof(float2))) ||
      (rc = p->f_torus.alloc((size_t)2 * L * L * sizeof(float2))) ||
      (rc = p->f_pad.alloc((size_t)4 * L * L * sizeof(float2))) ||
      (rc = p->f_synth.alloc((size_t)kFields * (L + 1) * (L + 1) * sizeof(float2))) ||
      (rc = p->f_samples.alloc((size_t)kFields * (L + 1) * 2 * L * sizeof(float))) ||
      (rc = p->f_jets.alloc((size_t)12 * (2 + (size_t)(L - 1) * 2 * L) * sizeof(float))))
    return rc;
  int n2[1] = {2 * L}, n4[1] = {4 * L};
  int inemb[1] = {2 * L}, onemb[1] = {L + 1}, tn[1] = {2 * L}, pn[1] = {4 * L};
  int cin[1] = {L + 1}, rout[1] = {2 * L};
  cufftResult r = cufftPlanMany(&p->f_ring_fwd, 1, n2, inemb, 1, 2 * L, onemb, 1, L + 1, CUFFT_R2C, L + 1);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftPlanMany(f_ring_fwd)");
  p->have_fplans[0] = true;
  r = cufftPlanMany(&p->f_torus_fwd, 1, n2, tn, L, 1, tn, L, 1, CUFFT_C2C, L);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftPlanMany(f_torus_fwd)");
  p->have_fplans[1] = true;
  r = cufftPlanMany(&p->f_pad_inv, 1, n4, pn, L, 1, pn, L, 1, CUFFT_C2C, L);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftPlanMany(f_pad_inv)");
  p->have_fplans[2] = true;
  r = cufftPlanMany(&p->f_ring_inv, 1, n2, cin, 1, L + 1, rout, 1, 2 * L, CUFFT_C2R, kFields * (L + 1));
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftPlanMany(f_ring_inv)");
  p->have_fplans[3] = true;
  return CMM_OK;
}

// Split-BF16 forward transform up to the Legendre stage: the samples in
// FP32, the ring FFTs, the torus extension and the padded inverse
// transform -> p->f_pad (the analysis' input).
static int forward_rings_f32(cmm_sht* p, const double* samples, cudaStream_t s) {
  const int L = p->L;
  int rc;
  dim3 b(128), g1((L + 127) / 128, 2 * L), g2((L + 127) / 128, 4 * L);
  const int64_t ns = (int64_t)(L + 1) * 2 * L;
  to_float_kernel<<<(int)((ns + 255) / 256), 256, 0, s>>>(samples, ns, (float*)p->f_in.p);
  if ((rc = check_launch("to_float_kernel"))) return rc;
  cufftResult r = cufftExecR2C(p->f_ring_fwd, (cufftReal*)p->f_in.p, (cufftComplex*)p->f_spec.p);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftExecR2C");
  torus_kernel<float2><<<g1, b, 0, s>>>((const float2*)p->f_spec.p, L, (float2*)p->f_torus.p);
  if ((rc = check_launch("torus_kernel"))) return rc;
  r = cufftExecC2C(p->f_torus_fwd, (cufftComplex*)p->f_torus.p, (cufftComplex*)p->f_torus.p, CUFFT_FORWARD);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftExecC2C(torus)");
  pad_kernel<float2><<<g2, b, 0, s>>>((const float2*)p->f_torus.p, L, (float2*)p->f_pad.p);
  if ((rc = check_launch("pad_kernel"))) return rc;
  r = cufftExecC2C(p->f_pad_inv, (cufftComplex*)p->f_pad.p, (cufftComplex*)p->f_pad.p, CUFFT_INVERSE);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftExecC2C(pad)");
  return CMM_OK;
}

// samples (L+1, 2L) -> alm (m-major half layout) in p->alm or `out`.
int sht_forward(cmm_sht* p, const double* samples, double2* out, cudaStream_t s) {
  const int L = p->L;
  int rc = set_streams(p, s);
  if (rc) return rc;
  dim3 b(128), g1((L + 127) / 128, 2 * L);
  if (p->precision == CMM_SHT_SPLIT_BF16) {
    if ((rc = forward_rings_f32(p, samples, s))) return rc;
    return tc_analysis(p->tc, (const float2*)p->f_pad.p, (const double*)p->w_fine.p, out,
                       (int*)p->status.p, s);
  }
  cufftResult r = cufftExecD2Z(p->ring_fwd, (cufftDoubleReal*)samples, (cufftDoubleComplex*)p->spec.p);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftExecD2Z");
  torus_t_kernel<<<g1, b, 0, s>>>((const double2*)p->spec.p, L, (double2*)p->torus.p);
  if ((rc = check_launch("torus_t_kernel"))) return rc;
  r = cufftExecZ2Z(p->torus_fwd_t, (cufftDoubleComplex*)p->torus.p, (cufftDoubleComplex*)p->torus.p,
                   CUFFT_FORWARD);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftExecZ2Z(torus)");
  pad_t_kernel<<<dim3((4 * L + 127) / 128, L), b, 0, s>>>((const double2*)p->torus.p, L, (double2*)p->pad.p);
  if ((rc = check_launch("pad_t_kernel"))) return rc;
  r = cufftExecZ2Z(p->pad_inv_t, (cufftDoubleComplex*)p->pad.p, (cufftDoubleComplex*)p->pad.p, CUFFT_INVERSE);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftExecZ2Z(pad)");
  if (L + 1 > 8 * 256) {
    set_last_error("sht_forward: L too large for the analysis kernel");
    return CMM_ERR_UNSUPPORTED;
  }
  bool tab;
  if ((rc = ensure_tables(p, s, &tab))) return rc;
  if (tab) {
    analysis_tab_kernel<<<dim3(L, (L + kTabBlock - 1) / kTabBlock), kTabBlock, 0, s>>>(
        (const double2*)p->pad.p, L, (const double*)p->w_fine.p, (const double*)p->tab->a.p, out);
    return check_launch("analysis_tab_kernel");
  }
  analysis_kernel<<<L, 256, 0, s>>>((const double2*)p->pad.p, L, (const double*)p->w_fine.p,
                                    (const double*)p->ct_fine.p, (const double*)p->pmm_fine.p,
                                    (const double*)p->ra.p, (const double*)p->rb.p, out);
  return check_launch("analysis_kernel");
}

// nf fields (nf, L, L) m-major -> samples (nf, L+1, 2L).
int sht_inverse(cmm_sht* p, const double2* alm, int nf, double* samples, cudaStream_t s) {
  const int L = p->L;
  int rc = set_streams(p, s);
  if (rc) return rc;
  if (nf == kFields && p->precision == CMM_SHT_SPLIT_BF16) {
    // tensor-core synthesis into FP32 spectra, FP32 ring FFTs
    const int nrows = kFields * (L + 1);
    zero_nyquist_kernel<<<(nrows + 255) / 256, 256, 0, s>>>((float2*)p->f_synth.p, L, nrows);
    if ((rc = check_launch("zero_nyquist_kernel"))) return rc;
    if ((rc = tc_synthesis(p->tc, alm, (float2*)p->f_synth.p, (int*)p->status.p, s))) return rc;
    cufftResult r = cufftExecC2R(p->f_ring_inv, (cufftComplex*)p->f_synth.p, (cufftReal*)p->f_samples.p);
    if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftExecC2R");
    if (samples) {
      const int64_t ns = (int64_t)nf * (L + 1) * 2 * L;
      to_double_kernel<<<(int)((ns + 255) / 256), 256, 0, s>>>((const float*)p->f_samples.p, ns, samples);
      return check_launch("to_double_kernel");
    }
    return CMM_OK;
  }
  if ((rc = ensure_fp64_inverse(p))) return rc;
  double2* S = (double2*)p->synth.p;
  // all kFields spectra: the batched Z2D below transforms every row
  cudaError_t e = cudaMemsetAsync(S, 0, (size_t)kFields * (L + 1) * (L + 1) * sizeof(double2), s);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
  const int npair = L / 2 + 1;
  bool tab;
  if ((rc = ensure_tables(p, s, &tab))) return rc;
  if (tab && (nf == kFields || nf == 4 || nf == 1)) {
    const int G = nf == kFields ? 3 : 1;
    dim3 gt(L, (npair + kTabBlock - 1) / kTabBlock, nf / G);
    if (G == 3)
      synthesis_tab_kernel<3><<<gt, kTabBlock, 0, s>>>(alm, L, (const double*)p->tab->s.p, S);
    else
      synthesis_tab_kernel<1><<<gt, kTabBlock, 0, s>>>(alm, L, (const double*)p->tab->s.p, S);
    if ((rc = check_launch("synthesis_tab_kernel"))) return rc;
  } else {
  dim3 g(L, (npair + kSynthBlock - 1) / kSynthBlock);
  if (nf == kFields)
    synthesis_kernel<kFields><<<g, kSynthBlock, 0, s>>>(alm, L, (const double*)p->ct_rings.p,
                                                        (const double*)p->pmm_rings.p,
                                                        (const double*)p->ra.p, (const double*)p->rb.p, S);
  else if (nf == 1)
    synthesis_kernel<1><<<g, kSynthBlock, 0, s>>>(alm, L, (const double*)p->ct_rings.p,
                                                  (const double*)p->pmm_rings.p, (const double*)p->ra.p,
                                                  (const double*)p->rb.p, S);
  else if (nf == 4)
    synthesis_kernel<4><<<g, kSynthBlock, 0, s>>>(alm, L, (const double*)p->ct_rings.p,
                                                  (const double*)p->pmm_rings.p, (const double*)p->ra.p,
                                                  (const double*)p->rb.p, S);
  else {
    set_last_error("sht_inverse: nf must be 1, 4 or 12");
    return CMM_ERR_ARG;
  }
  if ((rc = check_launch("synthesis_kernel"))) return rc;
  }
  // Z2D over kFields*(L+1) rows; only the first nf*(L+1) rows matter
  cufftResult r = cufftExecZ2D(p->ring_inv, (cufftDoubleComplex*)S, (cufftDoubleReal*)p->samples.p);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftExecZ2D");
  if (samples && samples != p->samples.p) {
    e = cudaMemcpyAsync(samples, p->samples.p, (size_t)nf * (L + 1) * 2 * L * 8, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync");
  }
  return CMM_OK;
}

// The stream function's 12 velocity/jet fields, their synthesis and the
// jets at the velocity mesh's vertices.
static int velocity_from_psi(cmm_sht* p, const cmm_mesh* vm, const double2* psi, double* jets,
                             cudaStream_t s);

int sht_velocity(cmm_sht* p, const cmm_mesh* vm, const double* omega, double2* psi_out,
                 double* jets, cudaStream_t s) {
  const int L = p->L;
  double2* psi = (double2*)p->alm.p;
  int rc;
  dim3 b(128), g((L + 127) / 128, L);
  if (omega) {
    if ((rc = sht_forward(p, omega, psi, s))) return rc;
    dinv_kernel<<<g, b, 0, s>>>(psi, L);
    if ((rc = check_launch("dinv_kernel"))) return rc;
    if (psi_out) {
      cudaError_t e = cudaMemcpyAsync(psi_out, psi, (size_t)L * L * sizeof(double2), cudaMemcpyDeviceToDevice, s);
      if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(psi)");
    }
  } else {
    psi = psi_out;  // stream function given by the caller
  }
  return velocity_from_psi(p, vm, psi, jets, s);
}

// Batched form of sht_velocity(p, vm, omega, NULL, jets): the forward
// transform up to the member's data tiles in its batch slot ...
int sht_velocity_pre(cmm_sht* p, const double* omega, cudaStream_t s) {
  if (!p->batch || p->precision != CMM_SHT_SPLIT_BF16 || !p->tc) {
    set_last_error("sht velocity (batched): a split-BF16 plan in a batch expected");
    return CMM_ERR_ARG;
  }
  int rc = set_streams(p, s);
  if (rc) return rc;
  if ((rc = forward_rings_f32(p, omega, s))) return rc;
  return tc_analysis_tiles(p->tc, (const float2*)p->f_pad.p, (const double*)p->w_fine.p,
                           (unsigned char*)p->batch->xtab.p, p->slot, s);
}

// ... and after the batch's analysis (which wrote p->alm), the rest.
int sht_velocity_post(cmm_sht* p, const cmm_mesh* vm, double* jets, cudaStream_t s) {
  const int L = p->L;
  int rc = set_streams(p, s);
  if (rc) return rc;
  double2* psi = (double2*)p->alm.p;
  dinv_kernel<<<dim3((L + 127) / 128, L), 128, 0, s>>>(psi, L);
  if ((rc = check_launch("dinv_kernel"))) return rc;
  return velocity_from_psi(p, vm, psi, jets, s);
}

int sht_batch_create(cmm_sht* const* plans, int n, cmm_sht_batch** out) {
  if (!plans || !out || n < 1 || n > 8) {
    set_last_error("cmm_sht_batch_create: 1 to 8 plans expected");
    return CMM_ERR_ARG;
  }
  for (int b = 0; b < n; ++b) {
    cmm_sht* p = plans[b];
    if (!p || p->L != plans[0]->L || p->precision != CMM_SHT_SPLIT_BF16 || !p->tc || p->batch) {
      set_last_error("cmm_sht_batch_create: distinct split-BF16 plans of one band-limit, in no other batch, "
                     "expected");
      return CMM_ERR_ARG;
    }
    for (int c = 0; c < b; ++c)
      if (plans[c] == p) {
        set_last_error("cmm_sht_batch_create: a plan appears twice");
        return CMM_ERR_ARG;
      }
  }
  cmm_sht_batch* bt = new (std::nothrow) cmm_sht_batch();
  if (!bt) {
    set_last_error("cmm_sht_batch_create: out of host memory");
    return CMM_ERR_NOMEM;
  }
  bt->L = plans[0]->L;
  bt->n = n;
  int rc = bt->xtab.alloc(tc_xtab_bytes(plans[0]->tc));
  if (rc) {
    delete bt;
    return rc;
  }
  cudaError_t e = cudaMemset(bt->xtab.p, 0, bt->xtab.bytes);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    delete bt;
    return cuda_fail(e, "cmm_sht_batch_create");
  }
  for (int b = 0; b < n; ++b) {
    bt->plans[b] = plans[b];
    plans[b]->batch = bt;
    plans[b]->slot = b;
  }
  *out = bt;
  return CMM_OK;
}

int sht_batch_size(const cmm_sht_batch* bt) { return bt->n; }

int sht_batch_destroy(cmm_sht_batch* bt) {
  if (!bt) return CMM_OK;
  cudaError_t e = cudaDeviceSynchronize();
  for (int b = 0; b < bt->n; ++b)
    if (bt->plans[b]) {
      bt->plans[b]->batch = nullptr;
      bt->plans[b]->slot = -1;
    }
  delete bt;
  return e == cudaSuccess ? CMM_OK : cuda_fail(e, "cmm_sht_batch_destroy");
}

// The batch's analysis into each member's own coefficients (out NULL) or
// into out[b].
int sht_batch_analysis(cmm_sht_batch* bt, double2* const* out, cudaStream_t s) {
  double2* alm[8];
  for (int b = 0; b < bt->n; ++b) {
    cmm_sht* p = bt->plans[b];
    if (!p || p->precision != CMM_SHT_SPLIT_BF16 || !p->tc || p->L != bt->L) {
      set_last_error("cmm_sht_batch_analysis: a member plan was destroyed or is no longer split-BF16");
      return CMM_ERR_ARG;
    }
    alm[b] = out ? out[b] : (double2*)p->alm.p;
  }
  return tc_analysis_batch(bt->plans[0]->tc, (const unsigned char*)bt->xtab.p, alm, bt->n,
                           (int*)bt->plans[0]->status.p, s);
}

// Forward transforms of one field per member: each member's rings and data
// tiles, then one batched analysis -> alm[b].
int sht_batch_forward(cmm_sht_batch* bt, const double* const* samples, double2* const* alm, cudaStream_t s) {
  for (int b = 0; b < bt->n; ++b) {
    cmm_sht* p = bt->plans[b];
    if (!p) {
      set_last_error("cmm_sht_batch_forward: a member plan was destroyed");
      return CMM_ERR_ARG;
    }
    int rc = sht_velocity_pre(p, samples[b], s);
    if (rc) return rc;
  }
  return sht_batch_analysis(bt, alm, s);
}

static int velocity_from_psi(cmm_sht* p, const cmm_mesh* vm, const double2* psi, double* jets,
                             cudaStream_t s) {
  const int L = p->L;
  int rc;
  dim3 b(128), g((L + 127) / 128, L);
  double2* F = (double2*)p->fields.p;
  ladder1_kernel<<<g, b, 0, s>>>(psi, L, F);
  if ((rc = check_launch("ladder1_kernel"))) return rc;
  ladder2_kernel<<<g, b, 0, s>>>(F, L);
  if ((rc = check_launch("ladder2_kernel"))) return rc;
  if ((rc = sht_inverse(p, F, kFields, nullptr, s))) return rc;
  const int64_t nv = 2 + (int64_t)(L - 1) * 2 * L;
  if (p->precision == CMM_SHT_SPLIT_BF16)
    jets_kernel<float><<<(int)((nv + 127) / 128), 128, 0, s>>>((const float*)p->f_samples.p, L,
                                                                vm->view.grid, jets, (float*)p->f_jets.p);
  else
    jets_kernel<double><<<(int)((nv + 127) / 128), 128, 0, s>>>((const double*)p->samples.p, L,
                                                                 vm->view.grid, jets, nullptr);
  return check_launch("jets_kernel");
}

// Transpose of sht_velocity (omega -> velocity jets, FP64 form):
// grad_jets (3,4,Nv_u) -> grad_omega (L+1, 2L), overwritten.
int sht_velocity_bwd(cmm_sht* p, const cmm_mesh* vm, const double* gjets, double* gomega,
                     cudaStream_t s) {
  const int L = p->L;
  int rc;
  if ((rc = ensure_fp64_inverse(p))) return rc;
  if (!p->have_bplans) {
    int n2[1] = {2 * L}, inemb[1] = {2 * L}, onemb[1] = {L + 1}, cin[1] = {L + 1}, rout[1] = {2 * L};
    cufftResult r = cufftPlanMany(&p->b_ring_fwd12, 1, n2, inemb, 1, 2 * L, onemb, 1, L + 1, CUFFT_D2Z,
                                  kFields * (L + 1));
    if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftPlanMany(b_ring_fwd12)");
    r = cufftPlanMany(&p->b_ring_inv1, 1, n2, cin, 1, L + 1, rout, 1, 2 * L, CUFFT_Z2D, L + 1);
    if (r != CUFFT_SUCCESS) {
      cufftDestroy(p->b_ring_fwd12);
      return cufft_fail(r, "cufftPlanMany(b_ring_inv1)");
    }
    p->have_bplans = true;
  }
  if ((rc = set_streams(p, s))) return rc;
  cufftResult r = cufftSetStream(p->b_ring_fwd12, s);
  if (r == CUFFT_SUCCESS) r = cufftSetStream(p->b_ring_inv1, s);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftSetStream");
  double* gf = (double*)p->samples.p;             // (12, L+1, 2L)
  double2* Sb = (double2*)p->synth.p;             // (12, L+1, L+1)
  double2* Fb = (double2*)p->fields.p;            // (12, L, L)
  double2* ab = (double2*)p->alm.p;               // (L, L)
  const size_t fsz = (size_t)kFields * (L + 1) * 2 * L * sizeof(double);
  cudaError_t e = cudaMemsetAsync(gf, 0, fsz, s);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
  const int64_t nv = 2 + (int64_t)(L - 1) * 2 * L;
  jets_bwd_kernel<<<(int)((nv + 127) / 128), 128, 0, s>>>(gjets, L, vm->view.grid, gf);
  if ((rc = check_launch("jets_bwd_kernel"))) return rc;
  // C2R^T: spectra = c_m D2Z(samples)
  r = cufftExecD2Z(p->b_ring_fwd12, (cufftDoubleReal*)gf, (cufftDoubleComplex*)Sb);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftExecD2Z(adjoint)");
  // synthesis^T: unit-weight Legendre sums over the L+1 rings, c_m = 2 for m > 0
  {
    const int npair = L / 2 + 1;
    const dim3 gl(L, kFields);
    const int64_t fin = (int64_t)(L + 1) * (L + 1), fout = (int64_t)L * L;
    const double* ct = (const double*)p->ct_rings.p;
    const double* pm = (const double*)p->pmm_rings.p;
    const double* ra = (const double*)p->ra.p;
    const double* rb = (const double*)p->rb.p;
    bool tab;
    if ((rc = ensure_tables(p, s, &tab))) return rc;
    if (tab) {
      const dim3 gt(L, (L + kTabBlock - 1) / kTabBlock, kFields / 2);
      legendre_sum_tab_kernel<2><<<gt, kTabBlock, 0, s>>>(Sb, L + 1, L, 2.0, (const double*)p->tab->s.p, Fb, fin,
                                                          fout);
    } else if (npair <= 256)
      legendre_sum_kernel<1><<<gl, 256, 0, s>>>(Sb, L + 1, L, L, nullptr, 2.0, ct, pm, L + 1, ra, rb, Fb, fin, fout);
    else if (npair <= 512)
      legendre_sum_kernel<2><<<gl, 256, 0, s>>>(Sb, L + 1, L, L, nullptr, 2.0, ct, pm, L + 1, ra, rb, Fb, fin, fout);
    else if (npair <= 1024)
      legendre_sum_kernel<4><<<gl, 256, 0, s>>>(Sb, L + 1, L, L, nullptr, 2.0, ct, pm, L + 1, ra, rb, Fb, fin, fout);
    else
      legendre_sum_kernel<8><<<gl, 256, 0, s>>>(Sb, L + 1, L, L, nullptr, 2.0, ct, pm, L + 1, ra, rb, Fb, fin, fout);
    if ((rc = check_launch("legendre_sum_kernel"))) return rc;
  }
  dim3 b(128), g((L + 127) / 128, L);
  ladder2_bwd_kernel<<<g, b, 0, s>>>(Fb, L);
  if ((rc = check_launch("ladder2_bwd_kernel"))) return rc;
  ladder1_bwd_kernel<<<g, b, 0, s>>>(Fb, L, ab);
  if ((rc = check_launch("ladder1_bwd_kernel"))) return rc;
  dinv_kernel<<<g, b, 0, s>>>(ab, L);
  if ((rc = check_launch("dinv_kernel"))) return rc;
  // analysis^T: weighted synthesis on the 2L+1 fine rings
  double2* H = (double2*)p->pad.p;                 // (4L, L)
  e = cudaMemsetAsync(H, 0, (size_t)4 * L * L * sizeof(double2), s);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
  const int nfp = L + 1;   // ring pairs of the fine grid (nr = 2L)
  ring_synthesis_kernel<<<dim3(L, (nfp + kSynthBlock - 1) / kSynthBlock), kSynthBlock, 0, s>>>(
      ab, L, 2 * L, (const double*)p->w_fine.p, (const double*)p->ct_fine.p, (const double*)p->pmm_fine.p,
      2 * L + 1, (const double*)p->ra.p, (const double*)p->rb.p, H, L);
  if ((rc = check_launch("ring_synthesis_kernel"))) return rc;
  // (Z2Z inverse 4L)^T = Z2Z forward 4L
  r = cufftExecZ2Z(p->pad_inv, (cufftDoubleComplex*)H, (cufftDoubleComplex*)H, CUFFT_FORWARD);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftExecZ2Z(adjoint pad)");
  double2* Gb = (double2*)p->torus.p;              // (2L, L)
  pad_bwd_kernel<<<dim3((L + 127) / 128, 2 * L), b, 0, s>>>(H, L, Gb);
  if ((rc = check_launch("pad_bwd_kernel"))) return rc;
  // (Z2Z forward 2L)^T = Z2Z inverse 2L
  r = cufftExecZ2Z(p->torus_fwd, (cufftDoubleComplex*)Gb, (cufftDoubleComplex*)Gb, CUFFT_INVERSE);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftExecZ2Z(adjoint torus)");
  double2* X = (double2*)p->spec.p;                // (L+1, L+1)
  torus_bwd_kernel<<<dim3((L + 1 + 127) / 128, L + 1), b, 0, s>>>(Gb, L, X);
  if ((rc = check_launch("torus_bwd_kernel"))) return rc;
  // D2Z^T: omega_bar[p] = Re sum_m specb_m e^{i m phi_p} (C2R of the prepared spectra)
  r = cufftExecZ2D(p->b_ring_inv1, (cufftDoubleComplex*)X, (cufftDoubleReal*)gomega);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftExecZ2D(adjoint)");
  return CMM_OK;
}

int sht_power(cmm_sht* p, const double2* alm, double* power, cudaStream_t s) {
  power_kernel<<<p->L, 256, 0, s>>>(alm, p->L, power);
  return check_launch("power_kernel");
}

int sht_scalar_jets(cmm_sht* p, const cmm_mesh* vm, const double2* alm, double* jets, cudaStream_t s) {
  const int L = p->L;
  double2* F = (double2*)p->fields.p;
  dim3 b(128), g((L + 127) / 128, L);
  scalar_fields_kernel<<<g, b, 0, s>>>(alm, L, F);
  int rc = check_launch("scalar_fields_kernel");
  if (rc) return rc;
  if ((rc = sht_inverse(p, F, 4, nullptr, s))) return rc;
  const int64_t nv = 2 + (int64_t)(L - 1) * 2 * L;
  scalar_jets_kernel<<<(int)((nv + 127) / 128), 128, 0, s>>>((const double*)p->samples.p, L,
                                                             vm->view.grid, jets);
  return check_launch("scalar_jets_kernel");
}

int sht_set_schedule(cmm_sht* p, int schedule) {
  if (schedule != 0 && schedule != 1) {
    set_last_error("cmm_sht_set_schedule: schedule 0 or 1 expected");
    return CMM_ERR_ARG;
  }
  p->tc_schedule = schedule;
  if (p->tc) tc_set_schedule(p->tc, schedule);
  return CMM_OK;
}

int sht_set_precision(cmm_sht* p, int mode) {
  if (mode != CMM_SHT_FP64 && mode != CMM_SHT_SPLIT_BF16) {
    set_last_error("cmm_sht_set_precision: unknown mode");
    return CMM_ERR_ARG;
  }
  if (mode == CMM_SHT_SPLIT_BF16 && !p->tc) {
    int rc = tc_plan_create(p->L, (const double*)p->ct_rings.p, (const double*)p->pmm_rings.p,
                            (const double*)p->ct_fine.p, (const double*)p->pmm_fine.p,
                            (const double*)p->ra.p, (const double*)p->rb.p, &p->tc);
    if (rc) return rc;
    tc_set_schedule(p->tc, p->tc_schedule);
    if (!p->have_fplans[0] && (rc = make_float_plans(p))) return rc;
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_fail(e, "cmm_sht_set_precision");
  }
  p->precision = mode;
  return CMM_OK;
}

int sht_set_tables(cmm_sht* p, int mode) {
  if (mode < -1 || mode > 1) {
    set_last_error("cmm_sht_set_tables: mode must be -1, 0 or 1");
    return CMM_ERR_ARG;
  }
  if (mode == 1 && p->L > kTabShared) {
    set_last_error("cmm_sht_set_tables: FP64 Pbar tables are limited to L <= 1024");
    return CMM_ERR_UNSUPPORTED;
  }
  p->tab_mode = mode;
  if (mode < 0 || (mode == 0 && p->L > kTabMaxL)) {
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_fail(e, "cmm_sht_set_tables");
    p->tab.reset();
  }
  return CMM_OK;
}

int sht_share_tables(cmm_sht* p, cmm_sht* src) {
  if (src->L != p->L || p == src) {
    set_last_error("cmm_sht_share_tables: a different source plan of the same L expected");
    return CMM_ERR_ARG;
  }
  if (src->precision == CMM_SHT_FP64) {
    // the FP64 Pbar tables, built on the source first when its table mode
    // gives it tables; p keeps its precision and takes src's table mode
    bool ok = false;
    int rc = ensure_tables(src, 0, &ok);
    cudaError_t e = cudaDeviceSynchronize();
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "cmm_sht_share_tables");
    if (!ok) {
      set_last_error("cmm_sht_share_tables: the source plan's FP64 stages run without Pbar tables");
      return CMM_ERR_ARG;
    }
    p->tab = src->tab;
    p->tab_mode = src->tab_mode;
    return CMM_OK;
  }
  if (!src->tc) {
    set_last_error("cmm_sht_share_tables: source plan without split-BF16 tables");
    return CMM_ERR_ARG;
  }
  if (p->tc) {
    tc_plan_destroy(p->tc);
    p->tc = nullptr;
  }
  int rc = tc_plan_share(src->tc, &p->tc);
  if (!rc) tc_set_schedule(p->tc, p->tc_schedule);
  if (rc) return rc;
  if (!p->have_fplans[0] && (rc = make_float_plans(p))) return rc;
  p->precision = CMM_SHT_SPLIT_BF16;
  cudaError_t e = cudaDeviceSynchronize();
  return e == cudaSuccess ? CMM_OK : cuda_fail(e, "cmm_sht_share_tables");
}

int sht_trim(cmm_sht* p) {
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_fail(e, "cmm_sht_trim");
  p->synth.release();
  p->samples.release();
  p->tab.reset();
  return CMM_OK;
}

int* sht_status_word(cmm_sht* p) { return (int*)p->status.p; }

int sht_status(cmm_sht* p, cudaStream_t s, int* flags, int clear) {
  int h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, p->status.p, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "cmm_sht_status");
  *flags = h;
  if (clear) {
    e = cudaMemsetAsync(p->status.p, 0, sizeof(int), s);
    if (e != cudaSuccess) return cuda_fail(e, "cmm_sht_status(clear)");
  }
  return CMM_OK;
}

int sht_destroy(cmm_sht* p) {
  delete p;
  return CMM_OK;
}

int sht_L(const cmm_sht* p) { return p->L; }

const float* sht_jets_f32(const cmm_sht* p) {
  return p->precision == CMM_SHT_SPLIT_BF16 && p->f_jets.p ? (const float*)p->f_jets.p : nullptr;
}

}  // namespace cmm
