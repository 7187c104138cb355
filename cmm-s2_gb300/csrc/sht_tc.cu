// Split-BF16 Legendre synthesis on the 5th-generation tensor cores
// (tcgen05, sm_103a).
//
// For each order m the inverse transform's Legendre stage is a product
//   S_even/odd[t][n] = sum_{l: l-m even/odd} Pbar_lm(theta_t) A[l][n]
// over ring pairs t (theta_t and pi - theta_t share |Pbar|; the parity of
// l-m gives the sign), with 24 real columns n (12 complex fields).  Each
// operand is split into two bf16 values, x = hi + lo (hi = bf16(x),
// lo = bf16(x - hi)), and the product is taken as three tensor-core
// products hi*hi + hi*lo + lo*hi accumulated in FP32 in tensor memory; the
// FP32 partial sums of every 64-l chunk are drained into compensated
// (Kahan) FP32 register sums, combined into the FP32 spectra at the end
// (FP64 issue would bind the kernel on GB300's FP64 pipe).
//
// Data movement: the Pbar tables (per m, ring block of 128 pairs, l chunk)
// are built once per plan directly in the shared-memory image the MMA
// reads (K-major, no swizzle, 8x8 core matrices of 128 bytes), so a chunk
// is one bulk asynchronous copy (cp.async.bulk) into shared memory.  One
// elected thread issues tcgen05.mma (M=128 ring pairs, N=32 columns,
// K=16) into two accumulators of 32 TMEM columns (even / odd l); all four
// warps read them back with tcgen05.ld.  Every wait on an mbarrier is
// bounded; on a timeout the kernel records CMM_FLAG_TIMEOUT, drains its own
// operations (a second bounded wait), releases its tensor memory and
// returns.
//
// The forward analysis f_lm = sum_j w_j Pbar_lm(theta'_j) F'_m(j) is the
// same contraction transposed: M = 128 degrees, N = 16 (re, im), K = 64
// fine ring pairs per chunk, with the quadrature weights and the ring-pair
// parity folding applied to the data tiles.
#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <memory>
#include <vector>

#include "cmm_internal.h"
#include "device_common.cuh"

namespace cmm {

namespace {

constexpr int kM = 128;                  // ring pairs per CTA (MMA M)
constexpr int kN = 32;                   // real columns per MMA (24 used)
constexpr int kNUsed = 24;
constexpr int kKc = 64;                  // l values per parity per chunk
constexpr int kPTile = kM * kKc * 2;     // bytes of one bf16 P tile = 16 KiB
constexpr int kATile = kN * kKc * 2;     // 4 KiB
constexpr int kPRecord = 4 * kPTile;     // E_hi, E_lo, O_hi, O_lo
constexpr int kARecord = 4 * kATile;
constexpr int kThreads = 128;
constexpr long long kSpinLimit = 1LL << 26;

// Byte offset of element (row, k) in a K-major no-swizzle tile image with
// 8x8 core matrices: core (row/8, k/8) at (row/8 * (K/8) + k/8) * 128,
// rows of 16 bytes inside.  Row-group stride (SBO) = (K/8) * 128 = 1024,
// k-group stride (LBO) = 128.
__host__ __device__ __forceinline__ int tile_offset(int row, int k) {
  return ((row >> 3) * (kKc >> 3) + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long limit = kSpinLimit) {
  for (long long i = 0; i < limit; ++i)
    if (mbar_test(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Compensated (Kahan) FP32 accumulation of the per-chunk partial sums:
// the running sum s and the negated lost low part c, sum = s - c.
struct KahanF {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
  __device__ __forceinline__ float valuef() const { return s - c; }
};

// Shared-memory matrix descriptor: start, leading (k-group) and stride
// (row-group) byte offsets, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((128u >> 4) & 0x3FFFu) << 16;    // LBO: next core matrix along K
  d |= (uint64_t)((1024u >> 4) & 0x3FFFu) << 32;   // SBO: next 8-row group
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::f16: D f32, A and B bf16, both K-major,
// N = 32, M = 128.
__device__ __forceinline__ uint32_t mma_idesc() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kN >> 3) << 17) | ((uint32_t)(kM >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

// 32 lanes x 32 consecutive 32-bit columns -> this thread's 32 values.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
        "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
        "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

struct TcGeometry {
  int L, npair, nrb;
  const int* cbase;   // (L+1) prefix sums of chunks per m
};

__device__ __forceinline__ int nchunks(int L, int m) {
  const int kmax = (L - m + 1) / 2;   // number of l with l - m even
  return (kmax + kKc - 1) / kKc;
}

// ---------------------------------------------------------------- tables
// One thread per (m, ring pair t): Pbar_lm(theta_t) for l = m..L-1 by the
// three-term recurrence in FP64, split into bf16 hi/lo, written into the
// tile images of record (m, chunk, ring block).
__global__ void build_ptab_kernel(TcGeometry g, const double* __restrict__ ct,
                                  const double* __restrict__ pmm, const double* __restrict__ ra,
                                  const double* __restrict__ rb, unsigned char* __restrict__ tab) {
  const int m = blockIdx.y;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int L = g.L;
  if (t >= g.nrb * kM) return;
  const int blk = t / kM, row = t % kM;
  const bool real_row = t < g.npair;
  const double x = real_row ? ct[t] : 0.0;
  double p0 = real_row ? pmm[(int64_t)m * (L + 1) + t] : 0.0, p1 = 0.0;
  // the table is zeroed at creation: padding rows and l >= L stay zero
  for (int l = m; l < L && real_row; ++l) {
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
    const int par = (l - m) & 1, j = (l - m) >> 1, c = j / kKc, k = j % kKc;
    unsigned char* rec = tab + ((int64_t)(g.cbase[m] + c) * g.nrb + blk) * kPRecord;
    const int off = tile_offset(row, k);
    const __nv_bfloat16 h = __double2bfloat16(P);
    const __nv_bfloat16 r = __double2bfloat16(P - (double)__bfloat162float(h));
    *(__nv_bfloat16*)(rec + (2 * par) * kPTile + off) = h;
    *(__nv_bfloat16*)(rec + (2 * par + 1) * kPTile + off) = r;
  }
}

// Per step: the 12 coefficient fields (12, L, L) [f][m][l] complex -> A tile
// images per (m, chunk): column n = 2f + (0 re, 1 im); columns n >= 24 are
// zeroed once when the plan is made and never written.
__global__ void build_atab_kernel(TcGeometry g, const double2* __restrict__ fields,
                                  unsigned char* __restrict__ atab) {
  const int m = blockIdx.y;
  const int L = g.L;
  const int nch = nchunks(L, m);
  const int per_chunk = 2 * kNUsed * kKc;   // (par, n < 24, k)
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nch * per_chunk; e += gridDim.x * blockDim.x) {
    const int c = e / per_chunk, r = e % per_chunk;
    const int par = r / (kNUsed * kKc), n = (r / kKc) % kNUsed, k = r % kKc;
    const int l = m + par + 2 * (c * kKc + k);
    float v = 0.f;
    if (l < L) {
      const double2 a = fields[(int64_t)(n >> 1) * L * L + (int64_t)m * L + l];
      v = dev::to_f32_trunc((n & 1) ? a.y : a.x);
    }
    // the split in FP32 from the coefficient truncated to FP32 (2^-23
    // relative, far inside the split's 2^-17): no FP64 pipe work
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    const __nv_bfloat16 lo = __float2bfloat16_rn(v - __bfloat162float(h));
    unsigned char* rec = atab + (int64_t)(g.cbase[m] + c) * kARecord;
    const int off = tile_offset(n, k);
    *(__nv_bfloat16*)(rec + (2 * par) * kATile + off) = h;
    *(__nv_bfloat16*)(rec + (2 * par + 1) * kATile + off) = lo;
  }
}

// ------------------------------------------------------------ synthesis
// Persistent: CTA b takes the work items (m, ring block) b, b + G, ... in
// order of increasing m (G = gridDim.x, one CTA per SM) and streams their
// l chunks through a two-stage pipeline: once the products of chunk k are
// in TMEM its stage is refilled with chunk k+2, chunk k+1 goes to the
// tensor cores (the other TMEM buffer), and all four warps drain chunk k
// into the compensated FP32 sums meanwhile.  Each work item
// writes its spectra S[f][t][m] for the ring pairs (t, L-t) of its rows
// after its last chunk.
constexpr int kSynStage = kPRecord + kARecord;   // 80 KiB per stage
constexpr uint32_t kTmemColsS = 128;             // 2 buffers x (even, odd) x 32 columns

struct SynCursor {
  int item, c, nch, m, blk;
};

// Cursor at work item `item`; false past the last one.
__device__ __forceinline__ bool syn_set(SynCursor& u, int item, int nitems, const TcGeometry& g) {
  u.item = item;
  u.c = 0;
  if (item >= nitems) return false;
  u.m = item / g.nrb;
  u.blk = item % g.nrb;
  u.nch = nchunks(g.L, u.m);
  return true;
}

// Next chunk of this CTA's stream; false at its end.
__device__ __forceinline__ bool syn_next(SynCursor& u, int nitems, const TcGeometry& g) {
  if (++u.c < u.nch) return true;
  return syn_set(u, u.item + gridDim.x, nitems, g);
}

__device__ __forceinline__ void syn_load(const TcGeometry& g, const unsigned char* ptab,
                                         const unsigned char* atab, const SynCursor& u, unsigned char* stage,
                                         uint64_t* bar) {
  const int64_t chunk = g.cbase[u.m] + u.c;
  const unsigned char* srcP = ptab + (chunk * g.nrb + u.blk) * kPRecord;
  const unsigned char* srcA = atab + chunk * kARecord;
  mbar_expect_tx(bar, kSynStage);
  for (int q = 0; q < 4; ++q) bulk_g2s(stage + q * kPTile, srcP + q * kPTile, kPTile, bar);
  bulk_g2s(stage + kPRecord, srcA, kARecord, bar);
}

// The chunk's products: even and odd l into the accumulators d, d + kN.
__device__ __forceinline__ void syn_mma(uint32_t stage, uint32_t d, uint32_t idesc) {
  const uint32_t p0 = stage, a0 = stage + kPRecord;
  for (int ks = 0; ks < kKc / 16; ++ks)
    for (int par = 0; par < 2; ++par) {
      const uint64_t ph = smem_desc(p0 + (2 * par) * kPTile + ks * 256);
      const uint64_t pl = smem_desc(p0 + (2 * par + 1) * kPTile + ks * 256);
      const uint64_t ah = smem_desc(a0 + (2 * par) * kATile + ks * 256);
      const uint64_t al = smem_desc(a0 + (2 * par + 1) * kATile + ks * 256);
      const uint32_t dd = d + par * kN;
      mma_bf16(dd, ph, ah, idesc, ks > 0 ? 1u : 0u);
      mma_bf16(dd, ph, al, idesc, 1u);
      mma_bf16(dd, pl, ah, idesc, 1u);
    }
}

__global__ void __launch_bounds__(kThreads, 1) synth_tc_kernel(TcGeometry g, int nitems,
                                                               const unsigned char* __restrict__ ptab,
                                                               const unsigned char* __restrict__ atab,
                                                               float2* __restrict__ S,
                                                               int* __restrict__ status) {
  extern __shared__ __align__(1024) unsigned char smem[];   // 2 stages of kSynStage bytes
  __shared__ __align__(8) uint64_t load_bar[2], mma_bar[2];
  __shared__ uint32_t tmem_base_s;
  __shared__ int abort_s;
  const int L = g.L;
  const int tid = threadIdx.x, warp = tid >> 5;
  if (tid == 0) {
    for (int b = 0; b < 2; ++b) {
      mbar_init(&load_bar[b], 1);
      mbar_init(&mma_bar[b], 1);
    }
    abort_s = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base_s)),
                 "r"(kTmemColsS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_s;
  const uint32_t idesc = mma_idesc();
  const uint32_t s0 = smem_u32(smem);
  SynCursor dr;   // next chunk to drain (all threads)
  bool have = syn_set(dr, blockIdx.x, nitems, g);
  // tid 0 only: next chunk to load / to multiply, and the chunk counts of
  // this CTA's stream issued and completed (chunk j uses stage and
  // barriers j & 1, in barrier phase (j >> 1) & 1)
  SynCursor ld = dr, mm = dr;
  bool ld_ok = have, mm_ok = have;
  long long n_ld = 0, n_ldw = 0, n_mm = 0, n_mmw = 0;
  if (tid == 0 && have) {
    for (int q = 0; q < 2 && ld_ok; ++q) {
      syn_load(g, ptab, atab, ld, smem + (n_ld & 1) * kSynStage, &load_bar[n_ld & 1]);
      ++n_ld;
      ld_ok = syn_next(ld, nitems, g);
    }
    if (!mbar_wait(&load_bar[0], 0)) {
      abort_s = 1;
    } else {
      n_ldw = 1;
      tc_fence_after();
      syn_mma(s0, tmem, idesc);
      mma_commit(&mma_bar[0]);
      n_mm = 1;
      mm_ok = syn_next(mm, nitems, g);
    }
  }
  KahanF accE[kNUsed], accO[kNUsed];
  __syncthreads();
  for (long long k = 0; have; ++k) {
    if (tid == 0 && !abort_s) {
      // chunk k's products (issued one iteration ago); its stage then takes
      // chunk k+2, so two copies are in flight while chunk k+1 arrives
      if (!mbar_wait(&mma_bar[k & 1], (uint32_t)((k >> 1) & 1))) {
        abort_s = 1;
      } else {
        n_mmw = k + 1;
        if (ld_ok) {
          syn_load(g, ptab, atab, ld, smem + (n_ld & 1) * kSynStage, &load_bar[n_ld & 1]);
          ++n_ld;
          ld_ok = syn_next(ld, nitems, g);
        }
      }
      if (!abort_s && mm_ok) {   // chunk k+1 (= n_mm) into the other TMEM buffer
        const int b1 = (int)(n_mm & 1);
        if (!mbar_wait(&load_bar[b1], (uint32_t)((n_mm >> 1) & 1))) {
          abort_s = 1;
        } else {
          n_ldw = n_mm + 1;
          tc_fence_after();
          syn_mma(s0 + b1 * kSynStage, tmem + b1 * 2 * kN, idesc);
          mma_commit(&mma_bar[b1]);
          ++n_mm;
          mm_ok = syn_next(mm, nitems, g);
        }
      }
    }
    __syncthreads();
    if (abort_s) break;
    tc_fence_after();
    float vE[32], vO[32];
    const uint32_t lanes = (uint32_t)(32 * warp) << 16;
    const uint32_t buf = tmem + (uint32_t)(k & 1) * 2 * kN;
    tmem_ld32(buf + lanes, vE);
    tmem_ld32(buf + lanes + kN, vO);
#pragma unroll
    for (int n = 0; n < kNUsed; ++n) {
      accE[n].add(vE[n]);
      accO[n].add(vO[n]);
    }
    if (dr.c == dr.nch - 1) {   // the work item's last chunk: its spectra
      const int t = dr.blk * kM + tid;   // TMEM lane = thread index
      if (t < g.npair) {
        // the spectra are FP32: the even/odd combination stays in FP32 (a
        // few ulp; FP64 here took 240 FP64-pipe operations per thread and
        // work item, the kernel's largest cost on GB300)
        const int64_t row_len = L + 1;
#pragma unroll
        for (int f = 0; f < kNUsed / 2; ++f) {
          const int64_t base = (int64_t)f * (L + 1) * row_len;
          const float eR = accE[2 * f].valuef(), eI = accE[2 * f + 1].valuef();
          const float oR = accO[2 * f].valuef(), oI = accO[2 * f + 1].valuef();
          S[base + (int64_t)t * row_len + dr.m] = make_float2(eR + oR, eI + oI);
          if (L - t != t) S[base + (int64_t)(L - t) * row_len + dr.m] = make_float2(eR - oR, eI - oI);
        }
      }
#pragma unroll
      for (int n = 0; n < kNUsed; ++n) accE[n] = accO[n] = KahanF();
    }
    tc_fence_before();
    __syncthreads();
    have = syn_next(dr, nitems, g);
  }
  if (tid == 0 && abort_s) {
    // bounded drain of this CTA's copies and products in flight
    bool drained = true;
    for (long long j = n_ldw; j < n_ld; ++j) drained &= mbar_wait(&load_bar[j & 1], (uint32_t)((j >> 1) & 1));
    for (long long j = n_mmw; j < n_mm; ++j) drained &= mbar_wait(&mma_bar[j & 1], (uint32_t)((j >> 1) & 1));
    atomicOr(status, drained ? CMM_FLAG_TIMEOUT : CMM_FLAG_TIMEOUT | CMM_FLAG_DRAIN_TIMEOUT);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemColsS)
                 : "memory");
}

// ------------------------------------------ synthesis, warp-specialised
// The same contraction and the same arithmetic as synth_tc_kernel (each
// 64-degree chunk's products accumulated in FP32 in tensor memory, the
// chunk partials summed in compensated FP32 registers), by three roles
// that run concurrently: warp 4 streams the chunks' tiles into a
// two-stage ring of shared memory (bulk copies), warp 5 issues each
// chunk's MMAs into one of two accumulator pairs as soon as its tiles have
// landed, and warps 0-3 (whose lanes are the 128 TMEM lanes, one ring pair
// each) add each chunk's partials into their compensated sums while the
// next chunk is multiplied into the other pair, writing a work item's
// spectra after its last chunk.  Stage and accumulator hand-offs go
// through mbarriers (copies complete `full`, MMA commits complete `empty`
// and `acc_full`, the four drain warps complete `acc_empty`); every wait
// is bounded and a timeout in any role stops all three.  The results are
// bitwise those of synth_tc_kernel.
constexpr int kSynWarps2 = 6;
constexpr int kSynStages2 = 2;

__device__ __forceinline__ bool wait_or_abort(uint64_t* bar, uint32_t parity, volatile int* abort) {
  for (long long i = 0; i < kSpinLimit; ++i) {
    if (mbar_test(bar, parity)) return true;
    if ((i & 255) == 255 && *abort) return false;
  }
  *abort = 1;
  return false;
}

__global__ void __launch_bounds__(32 * kSynWarps2, 1) synth_tc2_kernel(TcGeometry g, int nitems,
                                                                       const unsigned char* __restrict__ ptab,
                                                                       const unsigned char* __restrict__ atab,
                                                                       float2* __restrict__ S,
                                                                       int* __restrict__ status) {
  extern __shared__ __align__(1024) unsigned char smem[];   // kSynStages2 stages of kSynStage bytes
  __shared__ __align__(8) uint64_t full[kSynStages2], empty[kSynStages2], acc_full[2], acc_empty[2];
  __shared__ uint32_t tmem_base_s;
  __shared__ volatile int abort_s;
  __shared__ int drain_fail_s;
  const int L = g.L;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int b = 0; b < kSynStages2; ++b) {
      mbar_init(&full[b], 1);
      mbar_init(&empty[b], 1);
    }
    for (int a = 0; a < 2; ++a) {
      mbar_init(&acc_full[a], 1);
      mbar_init(&acc_empty[a], 4);
    }
    abort_s = 0;
    drain_fail_s = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base_s)),
                 "r"(kTmemColsS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_s;
  if (warp == 4 && lane == 0) {
    // producer: the tiles of every chunk of this CTA's items, in order
    long long j = 0;
    SynCursor u;
    bool ok = syn_set(u, blockIdx.x, nitems, g);
    while (ok && !abort_s) {
      const int st = (int)(j % kSynStages2);
      if (j >= kSynStages2 && !wait_or_abort(&empty[st], (uint32_t)((j / kSynStages2 - 1) & 1), &abort_s)) break;
      syn_load(g, ptab, atab, u, smem + st * kSynStage, &full[st]);
      ++j;
      ok = syn_next(u, nitems, g);
    }
    // copies still in flight land before the block exits: the stages'
    // last uses complete `full` (bounded)
    if (abort_s) {
      bool drained = true;
      for (long long k = (j > kSynStages2 ? j - kSynStages2 : 0); k < j; ++k)
        drained &= mbar_wait(&full[k % kSynStages2], (uint32_t)((k / kSynStages2) & 1));
      if (!drained) drain_fail_s = 1;
    }
  } else if (warp == 5 && lane == 0) {
    // MMA issuer: chunk j of this CTA's stream into accumulator pair j & 1
    const uint32_t idesc = mma_idesc();
    const uint32_t s0 = smem_u32(smem);
    long long j = 0;
    bool committed = false;
    SynCursor u;
    bool ok = syn_set(u, blockIdx.x, nitems, g);
    while (ok && !abort_s) {
      const int a = (int)(j & 1), st = (int)(j % kSynStages2);
      if (j >= 2 && !wait_or_abort(&acc_empty[a], (uint32_t)(((j >> 1) - 1) & 1), &abort_s)) break;
      if (!wait_or_abort(&full[st], (uint32_t)((j / kSynStages2) & 1), &abort_s)) break;
      tc_fence_after();
      syn_mma(s0 + st * kSynStage, tmem + a * 2 * kN, idesc);
      mma_commit(&empty[st]);
      mma_commit(&acc_full[a]);
      committed = true;
      ++j;
      ok = syn_next(u, nitems, g);
    }
    // products still in flight complete before the tensor memory is
    // released: the last commit's barrier (bounded)
    if (abort_s && committed) {
      const long long jl = j - 1;
      if (!mbar_wait(&empty[jl % kSynStages2], (uint32_t)((jl / kSynStages2) & 1))) drain_fail_s = 1;
    }
  } else if (warp < 4) {
    // drain: each chunk's partials into the compensated sums of the ring
    // pair (TMEM lane = thread index = ring row of the block), the spectra
    // after the item's last chunk
    KahanF accE[kNUsed], accO[kNUsed];
    long long j = 0;
    SynCursor dr;
    bool have = syn_set(dr, blockIdx.x, nitems, g);
    while (have) {
      const int a = (int)(j & 1);
      if (!wait_or_abort(&acc_full[a], (uint32_t)((j >> 1) & 1), &abort_s)) break;
      tc_fence_after();
      float vE[32], vO[32];
      const uint32_t lanes = (uint32_t)(32 * warp) << 16;
      const uint32_t buf = tmem + (uint32_t)a * 2 * kN;
      tmem_ld32(buf + lanes, vE);
      tmem_ld32(buf + lanes + kN, vO);
      tc_fence_before();
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&acc_empty[a])) : "memory");
#pragma unroll
      for (int n = 0; n < kNUsed; ++n) {
        accE[n].add(vE[n]);
        accO[n].add(vO[n]);
      }
      if (dr.c == dr.nch - 1) {   // the work item's last chunk: its spectra
        const int t = dr.blk * kM + tid;
        if (t < g.npair) {
          const int64_t row_len = L + 1;
#pragma unroll
          for (int f = 0; f < kNUsed / 2; ++f) {
            const int64_t base = (int64_t)f * (L + 1) * row_len;
            const float eR = accE[2 * f].valuef(), eI = accE[2 * f + 1].valuef();
            const float oR = accO[2 * f].valuef(), oI = accO[2 * f + 1].valuef();
            S[base + (int64_t)t * row_len + dr.m] = make_float2(eR + oR, eI + oI);
            if (L - t != t) S[base + (int64_t)(L - t) * row_len + dr.m] = make_float2(eR - oR, eI - oI);
          }
        }
#pragma unroll
        for (int n = 0; n < kNUsed; ++n) accE[n] = accO[n] = KahanF();
      }
      ++j;
      have = syn_next(dr, nitems, g);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (tid == 0 && abort_s) atomicOr(status, drain_fail_s ? CMM_FLAG_TIMEOUT | CMM_FLAG_DRAIN_TIMEOUT : CMM_FLAG_TIMEOUT);
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemColsS)
                 : "memory");
}

// -------------------------------------------------------------- analysis
// f_lm = sum_j Pbar_lm(theta'_j) X_par(l)[j] over the L+1 ring pairs j of
// the 2L+1 fine rings, X_even = w_j (F_j + F_{2L-j}), X_odd = w_j (F_j -
// F_{2L-j}) (ring L unpaired).  MMA rows are degrees l (128 per block, one
// parity per accumulator), columns the real and imaginary parts (N = 16,
// 2 used), K = 64 ring pairs per chunk.
constexpr int kNA = 16;
constexpr int kXTile = kNA * kKc * 2;        // 2 KiB
constexpr int kXRecord = 4 * kXTile;         // E_hi, E_lo, O_hi, O_lo
constexpr uint32_t kTmemColsA = 32;

struct TcFwdGeometry {
  int L, nck;           // ring-pair chunks of 64
  const int* lbase;     // (L+1) prefix sums of 128-degree blocks per m
};

__device__ __forceinline__ int nlblocks(int L, int m) {
  const int kmax = (L - m + 1) / 2;
  return (kmax + kM - 1) / kM;
}

__device__ __forceinline__ uint32_t mma_idesc_n16() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kNA >> 3) << 17) | ((uint32_t)(kM >> 4) << 24);
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// One thread per (m, fine ring pair j): Pbar_lm(theta'_j), l = m..L-1.
__global__ void build_ftab_kernel(TcFwdGeometry g, const double* __restrict__ ct,
                                  const double* __restrict__ pmm, const double* __restrict__ ra,
                                  const double* __restrict__ rb, unsigned char* __restrict__ tab) {
  const int m = blockIdx.y;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int L = g.L;
  if (j > L) return;   // pairs j = 0..L
  const double x = ct[j];
  double p0 = pmm[(int64_t)m * (2 * L + 1) + j], p1 = 0.0;
  const int c = j / kKc, k = j % kKc;
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
    const int par = (l - m) & 1, i = (l - m) >> 1, lb = i / kM, row = i % kM;
    unsigned char* rec = tab + ((int64_t)(g.lbase[m] + lb) * g.nck + c) * kPRecord;
    const int off = tile_offset(row, k);
    const __nv_bfloat16 h = __double2bfloat16(P);
    const __nv_bfloat16 r = __double2bfloat16(P - (double)__bfloat162float(h));
    *(__nv_bfloat16*)(rec + (2 * par) * kPTile + off) = h;
    *(__nv_bfloat16*)(rec + (2 * par + 1) * kPTile + off) = r;
  }
}

// Per transform: weighted, parity-folded fine-ring data -> X tile images
// per (m, ring chunk).  fine: (4L, L) FP32 complex [j][m] from the FP32
// ring FFTs, rows 0..2L used.
// slot: the field's column pair (2 slot, 2 slot + 1) of the 16-column data
// tiles (0 for a plan's own tiles; a batch's member index in shared tiles).
__global__ void build_xtab_kernel(TcFwdGeometry g, const float2* __restrict__ fine,
                                  const double* __restrict__ w, unsigned char* __restrict__ xtab,
                                  int slot) {
  const int m = blockIdx.y;
  const int L = g.L;
  // only the field's 2 columns (re, im); the other columns are zeroed once
  // when the tiles are made and written only by the other slots' fields
  const int total = g.nck * 2 * 2 * kKc;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const int c = e / (2 * 2 * kKc), r = e % (2 * 2 * kKc);
    const int par = r / (2 * kKc), n = (r / kKc) % 2, k = r % kKc;
    const int j = c * kKc + k;
    float v = 0.f;
    if (j <= L) {   // FP32 throughout: the samples are FP32, the split keeps 2^-17
      const float2 a = fine[(int64_t)j * L + m];
      float2 s;
      if (j < L) {
        const float2 b = fine[(int64_t)(2 * L - j) * L + m];
        s = par == 0 ? make_float2(a.x + b.x, a.y + b.y) : make_float2(a.x - b.x, a.y - b.y);
      } else {
        s = par == 0 ? a : make_float2(0.f, 0.f);
      }
      v = dev::to_f32_trunc(w[j]) * (n == 0 ? s.x : s.y);
    }
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    const __nv_bfloat16 lo = __float2bfloat16_rn(v - __bfloat162float(h));
    unsigned char* rec = xtab + ((int64_t)m * g.nck + c) * kXRecord;
    const int off = tile_offset(2 * slot + n, k);
    *(__nv_bfloat16*)(rec + (2 * par) * kXTile + off) = h;
    *(__nv_bfloat16*)(rec + (2 * par + 1) * kXTile + off) = lo;
  }
}

// Outputs of the analysis: field b (columns 2b, 2b + 1 of the data tiles)
// -> alm[b][m][l], b < n.
constexpr int kBatchMax = kNA / 2;
struct TcAlmOut {
  double2* p[kBatchMax];
  int n;
};

// Block (degree block, m); 128 threads; writes alm[b][m][l].  NB: column
// pairs drained (1 for a plan's own field; kBatchMax for a batch, whose
// fields share each Pbar tile the block streams).
template <int NB>
__global__ void __launch_bounds__(kThreads) analysis_tc_kernel(TcFwdGeometry g,
                                                               const unsigned char* __restrict__ ptab,
                                                               const unsigned char* __restrict__ xtab,
                                                               TcAlmOut out,
                                                               int* __restrict__ status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* sP = smem;                 // kPRecord
  unsigned char* sX = smem + kPRecord;      // kXRecord
  __shared__ __align__(8) uint64_t load_bar, mma_bar;
  __shared__ uint32_t tmem_base_s;
  __shared__ int abort_s;
  const int lb = blockIdx.x, m = blockIdx.y, L = g.L;
  if (lb >= nlblocks(L, m)) return;   // uniform for the block
  const int tid = threadIdx.x, warp = tid >> 5;
  if (tid == 0) {
    mbar_init(&load_bar, 1);
    mbar_init(&mma_bar, 1);
    abort_s = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base_s)),
                 "r"(kTmemColsA)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_s;
  const uint32_t idesc = mma_idesc_n16();
  KahanF aE[2 * NB], aO[2 * NB];
  uint32_t ph_load = 0, ph_mma = 0;
  for (int c = 0; c < g.nck; ++c) {
    if (tid == 0) {
      const unsigned char* srcP = ptab + ((int64_t)(g.lbase[m] + lb) * g.nck + c) * kPRecord;
      const unsigned char* srcX = xtab + ((int64_t)m * g.nck + c) * kXRecord;
      mbar_expect_tx(&load_bar, kPRecord + kXRecord);
      for (int q = 0; q < 4; ++q) bulk_g2s(sP + q * kPTile, srcP + q * kPTile, kPTile, &load_bar);
      bulk_g2s(sX, srcX, kXRecord, &load_bar);
      if (!mbar_wait(&load_bar, ph_load)) {
        abort_s = 1;
        if (!mbar_wait(&load_bar, ph_load)) abort_s = 2;   // bounded drain of the copies in flight
      }
      if (!abort_s) {
        tc_fence_after();
        const uint32_t p0 = smem_u32(sP), x0 = smem_u32(sX);
        for (int ks = 0; ks < kKc / 16; ++ks)
          for (int par = 0; par < 2; ++par) {
            const uint64_t ph = smem_desc(p0 + (2 * par) * kPTile + ks * 256);
            const uint64_t pl = smem_desc(p0 + (2 * par + 1) * kPTile + ks * 256);
            const uint64_t xh = smem_desc(x0 + (2 * par) * kXTile + ks * 256);
            const uint64_t xl = smem_desc(x0 + (2 * par + 1) * kXTile + ks * 256);
            const uint32_t d = tmem + par * kNA;
            mma_bf16(d, ph, xh, idesc, ks > 0 ? 1u : 0u);
            mma_bf16(d, ph, xl, idesc, 1u);
            mma_bf16(d, pl, xh, idesc, 1u);
          }
        mma_commit(&mma_bar);
        if (!mbar_wait(&mma_bar, ph_mma)) {
          abort_s = 1;
          if (!mbar_wait(&mma_bar, ph_mma)) abort_s = 2;   // bounded drain of the MMAs in flight
        }
      }
    }
    ph_load ^= 1u;
    ph_mma ^= 1u;
    __syncthreads();
    if (abort_s) break;
    tc_fence_after();
    float vE[16], vO[16];
    const uint32_t lane_base = (uint32_t)(32 * warp) << 16;
    tmem_ld16(tmem + lane_base, vE);
    tmem_ld16(tmem + lane_base + kNA, vO);
#pragma unroll
    for (int k = 0; k < 2 * NB; ++k) {
      aE[k].add(vE[k]);
      aO[k].add(vO[k]);
    }
    tc_fence_before();
    __syncthreads();
  }
  if (abort_s) {
    if (tid == 0) atomicOr(status, abort_s == 2 ? CMM_FLAG_TIMEOUT | CMM_FLAG_DRAIN_TIMEOUT : CMM_FLAG_TIMEOUT);
  } else {
    const int i = lb * kM + tid;
    const int lE = m + 2 * i, lO = m + 1 + 2 * i;
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      if (b >= out.n) break;
      double2* alm = out.p[b];
      if (lE < L) alm[(int64_t)m * L + lE] = make_double2(aE[2 * b].value(), aE[2 * b + 1].value());
      if (lO < L) alm[(int64_t)m * L + lO] = make_double2(aO[2 * b].value(), aO[2 * b + 1].value());
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemColsA)
                 : "memory");
}

int check(const char* what) {
  note_launch();
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? CMM_OK : cuda_fail(e, what);
}

}  // namespace

// Host side --------------------------------------------------------------
// The Pbar tables (read-only once built) may be shared by several plans
// of the same band-limit (tc_plan_share); the per-call data tiles atab /
// xtab are each plan's own, so plans sharing tables run concurrently.
struct TcTables {
  DeviceBuffer cbase, ptab, lbase, ftab;
};

struct TcPlan {
  int L = 0, npair = 0, nrb = 0, total_chunks = 0;
  int sms = 0;   // CTAs of the persistent synthesis (one per SM)
  int schedule = 1;   // synthesis: 1 warp-specialised (synth_tc2_kernel), 0 per-chunk drain
  // analysis: degree blocks of 128 per m (prefix sums), ring-pair chunks
  int nck = 0, total_lblocks = 0;
  std::shared_ptr<TcTables> tab;
  DeviceBuffer atab, xtab;
};

static int tc_chunks(int L, int m) {
  const int kmax = (L - m + 1) / 2;
  return (kmax + kKc - 1) / kKc;
}

int tc_plan_create(int L, const double* ct_rings, const double* pmm_rings, const double* ct_fine,
                   const double* pmm_fine, const double* ra, const double* rb, TcPlan** out) {
  TcPlan* p = new (std::nothrow) TcPlan();
  if (!p) {
    set_last_error("tc plan: out of host memory");
    return CMM_ERR_NOMEM;
  }
  p->tab = std::make_shared<TcTables>();
  p->L = L;
  p->npair = L / 2 + 1;
  p->nrb = (p->npair + kM - 1) / kM;
  std::vector<int> cb(L + 1, 0);
  for (int m = 0; m < L; ++m) cb[m + 1] = cb[m] + tc_chunks(L, m);
  p->total_chunks = cb[L];
  int rc;
  if ((rc = p->tab->cbase.upload(cb.data(), cb.size() * sizeof(int))) ||
      (rc = p->tab->ptab.alloc((size_t)p->total_chunks * p->nrb * kPRecord)) ||
      (rc = p->atab.alloc((size_t)p->total_chunks * kARecord))) {
    delete p;
    return rc;
  }
  cudaMemset(p->tab->ptab.p, 0, p->tab->ptab.bytes);
  cudaMemset(p->atab.p, 0, p->atab.bytes);
  TcGeometry g{L, p->npair, p->nrb, (const int*)p->tab->cbase.p};
  dim3 grid((p->nrb * kM + 127) / 128, L);
  build_ptab_kernel<<<grid, 128>>>(g, ct_rings, pmm_rings, ra, rb, (unsigned char*)p->tab->ptab.p);
  if ((rc = check("build_ptab_kernel"))) {
    delete p;
    return rc;
  }
  cudaError_t e = cudaFuncSetAttribute(synth_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       2 * kSynStage);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(synth_tc2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kSynStages2 * kSynStage);
  int dev = 0;
  if (e == cudaSuccess) e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) {
    delete p;
    return cuda_fail(e, "cudaFuncSetAttribute(synth_tc_kernel)");
  }
  // analysis tables over the L+1 fine ring pairs
  p->nck = (L + 1 + kKc - 1) / kKc;
  std::vector<int> lb(L + 1, 0);
  for (int m = 0; m < L; ++m) lb[m + 1] = lb[m] + ((L - m + 1) / 2 + kM - 1) / kM;
  p->total_lblocks = lb[L];
  if ((rc = p->tab->lbase.upload(lb.data(), lb.size() * sizeof(int))) ||
      (rc = p->tab->ftab.alloc((size_t)p->total_lblocks * p->nck * kPRecord)) ||
      (rc = p->xtab.alloc((size_t)L * p->nck * kXRecord))) {
    delete p;
    return rc;
  }
  cudaMemset(p->tab->ftab.p, 0, p->tab->ftab.bytes);
  cudaMemset(p->xtab.p, 0, p->xtab.bytes);
  TcFwdGeometry gf{L, p->nck, (const int*)p->tab->lbase.p};
  build_ftab_kernel<<<dim3((L + 1 + 127) / 128, L), 128>>>(gf, ct_fine, pmm_fine, ra, rb,
                                                            (unsigned char*)p->tab->ftab.p);
  if ((rc = check("build_ftab_kernel"))) {
    delete p;
    return rc;
  }
  e = cudaFuncSetAttribute(analysis_tc_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           kPRecord + kXRecord);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(analysis_tc_kernel<kBatchMax>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kPRecord + kXRecord);
  if (e != cudaSuccess) {
    delete p;
    return cuda_fail(e, "cudaFuncSetAttribute(analysis_tc_kernel)");
  }
  *out = p;
  return CMM_OK;
}

void tc_plan_destroy(TcPlan* p) { delete p; }

size_t tc_plan_bytes(const TcPlan* p) {
  return p->tab->ptab.bytes + p->atab.bytes + p->tab->ftab.bytes + p->xtab.bytes;
}

// A plan of the same band-limit using src's Pbar tables and its own tiles.
int tc_plan_share(const TcPlan* src, TcPlan** out) {
  TcPlan* p = new (std::nothrow) TcPlan();
  if (!p) {
    set_last_error("tc plan: out of host memory");
    return CMM_ERR_NOMEM;
  }
  p->L = src->L;
  p->npair = src->npair;
  p->nrb = src->nrb;
  p->sms = src->sms;
  p->total_chunks = src->total_chunks;
  p->nck = src->nck;
  p->total_lblocks = src->total_lblocks;
  p->tab = src->tab;
  int rc;
  if ((rc = p->atab.alloc(src->atab.bytes)) || (rc = p->xtab.alloc(src->xtab.bytes))) {
    delete p;
    return rc;
  }
  cudaError_t e = cudaMemset(p->atab.p, 0, p->atab.bytes);
  if (e == cudaSuccess) e = cudaMemset(p->xtab.p, 0, p->xtab.bytes);
  if (e != cudaSuccess) {
    delete p;
    return cuda_fail(e, "tc_plan_share");
  }
  *out = p;
  return CMM_OK;
}

namespace {

// Self-test of the timeout path: the tensor-core kernels' bounded wait on
// an mbarrier that no copy or MMA will ever complete (nothing arrives on
// it), with a limit of `polls`; on the timeout the block records
// CMM_FLAG_TIMEOUT in the status word and returns, as those kernels do.
__global__ void wait_timeout_probe_kernel(long long polls, int* __restrict__ status) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) mbar_init(&bar, 1);
  __syncthreads();
  const bool ok = mbar_wait(&bar, 0, polls);
  __syncthreads();
  if (threadIdx.x == 0 && !ok) atomicOr(status, CMM_FLAG_TIMEOUT);
}

}  // namespace

int tc_wait_timeout_probe(long long polls, int* status, cudaStream_t s) {
  wait_timeout_probe_kernel<<<1, 32, 0, s>>>(polls, status);
  return check("wait_timeout_probe_kernel");
}

void tc_set_schedule(TcPlan* p, int schedule) { p->schedule = schedule; }

int tc_synthesis(TcPlan* p, const double2* fields, float2* S, int* status, cudaStream_t s) {
  TcGeometry g{p->L, p->npair, p->nrb, (const int*)p->tab->cbase.p};
  build_atab_kernel<<<dim3(16, p->L), 256, 0, s>>>(g, fields, (unsigned char*)p->atab.p);
  int rc = check("build_atab_kernel");
  if (rc) return rc;
  const int nitems = p->L * p->nrb;
  const int grid = std::min(nitems, std::max(p->sms, 1));
  if (p->schedule == 1) {
    synth_tc2_kernel<<<grid, 32 * kSynWarps2, kSynStages2 * kSynStage, s>>>(
        g, nitems, (const unsigned char*)p->tab->ptab.p, (const unsigned char*)p->atab.p, S, status);
    return check("synth_tc2_kernel");
  }
  synth_tc_kernel<<<grid, kThreads, 2 * kSynStage, s>>>(
      g, nitems, (const unsigned char*)p->tab->ptab.p, (const unsigned char*)p->atab.p, S, status);
  return check("synth_tc_kernel");
}

// fine (4L, L) complex after the padded inverse transform, rows 0..2L;
// w the 2L+1 Clenshaw-Curtis weights -> alm[m][l], l >= m.
int tc_analysis(TcPlan* p, const float2* fine, const double* w, double2* alm, int* status,
                cudaStream_t s) {
  int rc = tc_analysis_tiles(p, fine, w, (unsigned char*)p->xtab.p, 0, s);
  if (rc) return rc;
  return tc_analysis_batch(p, (const unsigned char*)p->xtab.p, &alm, 1, status, s);
}

size_t tc_xtab_bytes(const TcPlan* p) { return p->xtab.bytes; }

int tc_analysis_tiles(TcPlan* p, const float2* fine, const double* w, unsigned char* xtab, int slot,
                      cudaStream_t s) {
  const int L = p->L;
  TcFwdGeometry g{L, p->nck, (const int*)p->tab->lbase.p};
  build_xtab_kernel<<<dim3(8, L), 256, 0, s>>>(g, fine, w, xtab, slot);
  return check("build_xtab_kernel");
}

int tc_analysis_batch(TcPlan* p, const unsigned char* xtab, double2* const* alm, int n, int* status,
                      cudaStream_t s) {
  if (n < 1 || n > kBatchMax) {
    set_last_error("tc analysis: 1 to 8 fields per launch");
    return CMM_ERR_ARG;
  }
  const int L = p->L;
  TcFwdGeometry g{L, p->nck, (const int*)p->tab->lbase.p};
  TcAlmOut out{};
  for (int b = 0; b < n; ++b) out.p[b] = alm[b];
  out.n = n;
  const int maxlb = ((L + 1) / 2 + kM - 1) / kM;
  if (n == 1)
    analysis_tc_kernel<1><<<dim3(maxlb, L), kThreads, kPRecord + kXRecord, s>>>(
        g, (const unsigned char*)p->tab->ftab.p, xtab, out, status);
  else
    analysis_tc_kernel<kBatchMax><<<dim3(maxlb, L), kThreads, kPRecord + kXRecord, s>>>(
        g, (const unsigned char*)p->tab->ftab.p, xtab, out, status);
  return check("analysis_tc_kernel");
}

}  // namespace cmm
