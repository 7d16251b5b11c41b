// Split-precision BF16 overlap matrices on the 5th-generation tensor
// cores: S = X^H Y for every k-set, X, Y complex64 [nb][npw].
//
// Real form: with the interleaved (re, im) coefficients as the contraction
// axis K = 2 npw,
//   Re S_ij = sum_K X_i[K] Y_j[K],   Im S_ij = sum_K X_i[K] (-i Y_j)[K]
// where (-i y) interleaves (y_im, -y_re).  One GEMM with A = X (M = 128 rows,
// bands padded) and B = [Y ; -iY] (N = 2 nb rounded to 16) yields both parts.
// Each FP32 operand is split into bf16 hi + lo, and the four products
// hi*hi + hi*lo + lo*hi + lo*lo accumulate in FP32 in tensor memory.  The
// lo*lo term is kept: on a Gram diagonal sum_K x_K^2 it has one sign for
// every K, so dropping it (the usual three-product split) biases |x|^2 low by
// about 2^-18 relative, which shows up as an excess electron count and a
// free-energy offset near 1e-6 Ha per electron; with it the remaining error
// (rounding of lo) has random sign.
//
// One CTA owns one k-set's K-range (split-K).  Per 64-element K block the
// 256 threads convert their share of X and Y into the canonical no-swizzle
// K-major core-matrix layout (8 rows x 16 bytes per core matrix), one thread
// issues the 16 tcgen05.mma (4 K-steps x 4 products) and commits them to the
// stage's mbarrier; two stages overlap conversion with the MMAs.  The
// accumulator is read back with tcgen05.ld and written as an FP64 partial
// that k_overlap_reduce sums over the splits.
//
// Every mbarrier wait is bounded; on timeout the CTA records
// DEREK_ERR_TIMEOUT, waits (bounded) for its own MMAs, frees its tensor
// memory and returns.
#include <cuda_bf16.h>

#include "subspace.cuh"

namespace derek {

namespace {

constexpr int TC_M = 128;
constexpr int TC_KB = 64;           // K elements (reals) per block
constexpr int TC_THREADS = 256;
constexpr long kWaitLimit = 1L << 26;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
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

__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, long limit = kWaitLimit) {
  for (long i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Try limit of the pipeline-stage waits (a stage is reused once the MMAs
// that read it completed).  The host lowers it to test the timeout path
// (derek_gpu_set_wait_limit); the final wait for a CTA's own MMAs, before it
// frees its tensor memory, always keeps the full kWaitLimit.
__device__ long g_stage_wait_limit = kWaitLimit;

// shared-memory matrix descriptor, no swizzle, K-major canonical layout:
// core matrices of 8 rows x 16 bytes; lbo = stride between core matrices
// along K, sbo = stride between 8-row groups.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version
  return d;                // layout type 0 = no swizzle
}

// instruction descriptor: kind::f16, A = B = bf16, D = f32, both K-major
__device__ __forceinline__ uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
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

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// byte offset of (row, k) inside a [rows][64] K-major no-swizzle tile
__device__ __forceinline__ uint32_t core_off(int row, int k8) {
  // core (row/8, k8) -> ((row/8)*8 + k8)*128, row%8 -> 16 B
  return (uint32_t)((((row >> 3) << 3) + k8) << 7) + (uint32_t)((row & 7) << 4);
}

__device__ __forceinline__ void split8(const float *v, uint4 &hi, uint4 &lo) {
  __nv_bfloat16 h[8], l[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    h[i] = __float2bfloat16_rn(v[i]);
    l[i] = __float2bfloat16_rn(v[i] - __bfloat162float(h[i]));
  }
  hi = *reinterpret_cast<uint4 *>(h);
  lo = *reinterpret_cast<uint4 *>(l);
}

}  // namespace

__global__ void __launch_bounds__(TC_THREADS, 1)
    k_overlap_tc(const Tables t, int ks_begin, const float2 *__restrict__ X, const float2 *__restrict__ Y,
                 double2 *__restrict__ part, const long long *__restrict__ part_off, int ksplit,
                 int *__restrict__ status) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bars[3];
  __shared__ uint32_t tmem_slot;
  __shared__ int s_ok;
  const int ksi = ks_begin + blockIdx.y;
  const KSetDev &K = t.ks[ksi];
  if (!t.sys[K.sys].active) return;
  const int split = blockIdx.x;
  const int g0 = split * ksplit;       // complex coefficients
  if (g0 >= K.npw) return;
  const int g1 = min(K.npw, g0 + ksplit);
  const int nb = K.nb;
  const int N = ((2 * nb + 15) / 16) * 16;
  const int tid = threadIdx.x, warp = tid >> 5;
  // stage layout: A_hi, A_lo (128 x 64 bf16 = 16 KB each), B_hi, B_lo (N x 64)
  const uint32_t a_bytes = TC_M * TC_KB * 2, b_bytes = (uint32_t)N * TC_KB * 2;
  const uint32_t stage_bytes = 2 * a_bytes + 2 * b_bytes;
  unsigned char *stage[2] = {smem_raw, smem_raw + stage_bytes};

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_slot)),
                 "r"(256)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_init(&bars[2], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = idesc_bf16(TC_M, N);

  const float *Xb = reinterpret_cast<const float *>(X + K.psi_off);
  const float *Yb = reinterpret_cast<const float *>(Y + K.psi_off);
  const long ld = 2L * K.npw_pad;  // floats per band row
  const int k0 = 2 * g0, k1 = 2 * g1;  // real K range
  const int nkb = (k1 - k0 + TC_KB - 1) / TC_KB;
  bool ok = true;

  // Jobs per K block: A rows j < nb (chunk (j, k8) of X) and B rows j < nb
  // (chunk (j, k8) of Y, which also gives row nb + j = -i Y_j); job q of
  // thread tid is c = tid + q TC_THREADS.  The raw chunks of the next K block
  // are loaded into registers while the current one is converted.
  constexpr int QJ = 2 * TC_M * 8 / TC_THREADS;   // jobs per thread at nb = 128
  // S = X^H X (Y == X): the A job's chunk also gives the B rows, so Y is not
  // loaded a second time
  const bool same = X == Y;
  const int njobs = (same ? 1 : 2) * nb * 8;
  // rows no job writes stay zero: A rows >= nb, B rows >= 2 nb (both stages)
  for (int s2 = 0; s2 < 2; ++s2) {
    unsigned char *A_hi = stage[s2], *A_lo = A_hi + a_bytes, *B_hi = A_lo + a_bytes,
                  *B_lo = B_hi + b_bytes;
    const uint4 z = make_uint4(0u, 0u, 0u, 0u);
    for (int c = tid; c < (TC_M - nb) * 8; c += TC_THREADS) {
      const int row = nb + (c >> 3), k8 = c & 7;
      *reinterpret_cast<uint4 *>(A_hi + core_off(row, k8)) = z;
      *reinterpret_cast<uint4 *>(A_lo + core_off(row, k8)) = z;
    }
    for (int c = tid; c < (N - 2 * nb) * 8; c += TC_THREADS) {
      const int row = 2 * nb + (c >> 3), k8 = c & 7;
      *reinterpret_cast<uint4 *>(B_hi + core_off(row, k8)) = z;
      *reinterpret_cast<uint4 *>(B_lo + core_off(row, k8)) = z;
    }
  }
  float4 nxt[QJ][2];
  auto load_block = [&](int kb) {
    const int kbase = k0 + kb * TC_KB;
#pragma unroll
    for (int q = 0; q < QJ; ++q) {
      const int c = tid + q * TC_THREADS;
      if (c < njobs) {
        const bool isB = c >= nb * 8;
        const int cc = isB ? c - nb * 8 : c;
        const int row = cc >> 3, k8 = cc & 7;
        const int kk = kbase + k8 * 8;
        const float *src = (isB ? Yb : Xb) + row * ld + kk;
        if (kk + 8 <= k1) {
          nxt[q][0] = *reinterpret_cast<const float4 *>(src);
          nxt[q][1] = *reinterpret_cast<const float4 *>(src + 4);
        } else {
          float w[8];
#pragma unroll
          for (int i = 0; i < 8; ++i) w[i] = kk + i < k1 ? src[i] : 0.0f;
          nxt[q][0] = make_float4(w[0], w[1], w[2], w[3]);
          nxt[q][1] = make_float4(w[4], w[5], w[6], w[7]);
        }
      }
    }
  };
  if (nkb > 0) load_block(0);

  for (int kb = 0; kb < nkb; ++kb) {
    const int s = kb & 1;
    if (kb >= 2) {
      // the MMAs of block kb-2 must have finished reading this stage
      if (tid == 0) s_ok = mbar_wait(&bars[s], ((kb - 2) >> 1) & 1, g_stage_wait_limit) ? 1 : 0;
      __syncthreads();
      if (!s_ok) {
        ok = false;
        break;
      }
    }
    unsigned char *A_hi = stage[s], *A_lo = A_hi + a_bytes, *B_hi = A_lo + a_bytes,
                  *B_lo = B_hi + b_bytes;
    float4 cur[QJ][2];
#pragma unroll
    for (int q = 0; q < QJ; ++q) {
      cur[q][0] = nxt[q][0];
      cur[q][1] = nxt[q][1];
    }
    if (kb + 1 < nkb) load_block(kb + 1);
#pragma unroll
    for (int q = 0; q < QJ; ++q) {
      const int c = tid + q * TC_THREADS;
      if (c < njobs) {
        const bool isB = c >= nb * 8;
        const int cc = isB ? c - nb * 8 : c;
        const int row = cc >> 3, k8 = cc & 7;
        const float v[8] = {cur[q][0].x, cur[q][0].y, cur[q][0].z, cur[q][0].w,
                            cur[q][1].x, cur[q][1].y, cur[q][1].z, cur[q][1].w};
        uint4 hi, lo;
        split8(v, hi, lo);
        if (!isB) {
          *reinterpret_cast<uint4 *>(A_hi + core_off(row, k8)) = hi;
          *reinterpret_cast<uint4 *>(A_lo + core_off(row, k8)) = lo;
          if (same) {
            *reinterpret_cast<uint4 *>(B_hi + core_off(row, k8)) = hi;
            *reinterpret_cast<uint4 *>(B_lo + core_off(row, k8)) = lo;
            const float w[8] = {v[1], -v[0], v[3], -v[2], v[5], -v[4], v[7], -v[6]};
            split8(w, hi, lo);
            *reinterpret_cast<uint4 *>(B_hi + core_off(nb + row, k8)) = hi;
            *reinterpret_cast<uint4 *>(B_lo + core_off(nb + row, k8)) = lo;
          }
        } else {
          *reinterpret_cast<uint4 *>(B_hi + core_off(row, k8)) = hi;
          *reinterpret_cast<uint4 *>(B_lo + core_off(row, k8)) = lo;
          // row nb + j: -i Y_j interleaves (y_im, -y_re)
          const float w[8] = {v[1], -v[0], v[3], -v[2], v[5], -v[4], v[7], -v[6]};
          split8(w, hi, lo);
          *reinterpret_cast<uint4 *>(B_hi + core_off(nb + row, k8)) = hi;
          *reinterpret_cast<uint4 *>(B_lo + core_off(nb + row, k8)) = lo;
        }
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t ah = smem_u32(A_hi), al = smem_u32(A_lo), bh = smem_u32(B_hi), bl = smem_u32(B_lo);
#pragma unroll
      for (int ks = 0; ks < TC_KB / 16; ++ks) {
        const uint32_t o = ks * 256;  // two core matrices along K per MMA
        const uint64_t dah = smem_desc(ah + o, 128, 1024), dal = smem_desc(al + o, 128, 1024);
        const uint64_t dbh = smem_desc(bh + o, 128, 1024), dbl = smem_desc(bl + o, 128, 1024);
        mma_bf16(tmem, dah, dbh, idesc, (kb > 0 || ks > 0) ? 1u : 0u);
        mma_bf16(tmem, dah, dbl, idesc, 1u);
        mma_bf16(tmem, dal, dbh, idesc, 1u);
        mma_bf16(tmem, dal, dbl, idesc, 1u);
      }
      mma_commit(&bars[s]);
    }
  }
  if (tid == 0) {
    mma_commit(&bars[2]);
    s_ok = mbar_wait(&bars[2], 0) ? 1 : 0;
  }
  __syncthreads();
  if (!s_ok) ok = false;
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok) {
    // accumulator: lane = row i, column = j; warps w and w+4 share lane quarter w%4
    const int quarter = warp & 3;
    const int half = warp >> 2;
    const int row = quarter * 32 + (tid & 31);
    const int ncol_half = N / 2;
    const int cbeg = half * ncol_half;
    double2 *P = part + part_off[ksi] + (long long)split * nb * nb;
    for (int c = cbeg; c < cbeg + ncol_half; c += 16) {
      uint32_t r[16];
      tmem_ld16(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)c, r);
      if (row < nb) {
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const int j = c + q;
          const double v = (double)__uint_as_float(r[q]);
          if (j < nb)
            reinterpret_cast<double *>(&P[row * nb + j])[0] = v;
          else if (j < 2 * nb)
            reinterpret_cast<double *>(&P[row * nb + (j - nb)])[1] = v;
        }
      }
    }
  } else if (tid == 0) {
    atomicExch(status + ksi, DEREK_ERR_TIMEOUT);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(256) : "memory");
  }
}

size_t overlap_tc_smem(int max_nb) {
  const int N = ((2 * max_nb + 15) / 16) * 16;
  return 2 * (2 * (size_t)TC_M * TC_KB * 2 + 2 * (size_t)N * TC_KB * 2);
}

void launch_overlap_tc(const Tables &t, int ks_begin, int nks, int max_nb, int max_npw, int ksplit,
                       const float2 *X, const float2 *Y, double2 *part, const long long *part_off,
                       double2 *out, const long long *mat_off, int hermitize, int *status,
                       cudaStream_t st) {
  if (nks <= 0) return;
  const size_t sm = overlap_tc_smem(max_nb);
  cudaFuncSetAttribute(k_overlap_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  dim3 grid((max_npw + ksplit - 1) / ksplit, nks);
  derek::note_launch(), k_overlap_tc<<<grid, TC_THREADS, sm, st>>>(t, ks_begin, X, Y, part, part_off, ksplit, status);
  launch_overlap_reduce(t, ks_begin, nks, part, part_off, ksplit, out, mat_off, hermitize, st);
}

}  // namespace derek

// ---------------------------------------------------------------------------
// Rotation X <- X C on the tensor cores (bf16 hi + lo split, four products),
// in place per 128-G tile.
//
// Real form per coefficient G: with x_G = (Re X_0, Im X_0, Re X_1, ...) the
// rotated row is y_G = M x_G, M = [[Re C, -Im C], [Im C, Re C]] per (i, j)
// block.  A = the tile's x_G rows (M = 128 G, K = 2 nb), B = M's rows
// (N = 2 nb): B[2j][2i] = Re C_ij, B[2j][2i+1] = -Im C_ij,
// B[2j+1][2i] = Im C_ij, B[2j+1][2i+1] = Re C_ij.  The accumulator row G,
// columns (2j, 2j+1) is the new coefficient X_j(G).
// ---------------------------------------------------------------------------
namespace derek {

namespace {
__device__ __forceinline__ void cp_async16_tc(void *smem, const void *gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(smem)), "l"(gmem) : "memory");
}
}  // namespace

// bytes of one k-set's B operand image: per K block, bf16 hi then lo of M's
// N rows in the core-matrix layout (2 x N x 64 x 2 bytes)
size_t rotate_tc_image_bytes(int max_nb) {
  const int N = ((2 * max_nb + 15) / 16) * 16;
  const int nkb = (2 * max_nb + TC_KB - 1) / TC_KB;
  return (size_t)nkb * 4 * N * TC_KB;
}

// The rotation's B operand (M built from the FP64 C) for every k-set,
// converted once here instead of in every 128-G tile of the rotation.
__global__ void __launch_bounds__(256) k_rotate_operand(const Tables t, int ks_begin, const double2 *__restrict__ C,
                                                        const long long *__restrict__ mat_off,
                                                        unsigned char *__restrict__ img, long long stride) {
  const int ksi = ks_begin + blockIdx.y;
  const KSetDev &K = t.ks[ksi];
  if (!t.sys[K.sys].active) return;
  const int nb = K.nb;
  const int N = ((2 * nb + 15) / 16) * 16;
  const int nkb = (2 * nb + TC_KB - 1) / TC_KB;
  const double2 *Cb = C + mat_off[ksi];
  unsigned char *base = img + (long long)blockIdx.y * stride;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nkb * N * 8; c += gridDim.x * blockDim.x) {
    const int kb = c / (N * 8), rem = c - kb * (N * 8);
    const int row = rem >> 3, k8 = rem & 7;
    const int j = row >> 1, part = row & 1;
    const int ib = kb * (TC_KB / 2);
    float v[8];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i = ib + 4 * k8 + q;
      double2 cij = make_double2(0.0, 0.0);
      if (row < 2 * nb && i < nb) cij = Cb[(long long)i * nb + j];
      if (part == 0) {
        v[2 * q] = (float)cij.x;
        v[2 * q + 1] = (float)(-cij.y);
      } else {
        v[2 * q] = (float)cij.y;
        v[2 * q + 1] = (float)cij.x;
      }
    }
    uint4 hi, lo;
    split8(v, hi, lo);
    unsigned char *blk = base + (size_t)kb * 4 * N * TC_KB;
    *reinterpret_cast<uint4 *>(blk + core_off(row, k8)) = hi;
    *reinterpret_cast<uint4 *>(blk + (size_t)2 * N * TC_KB + core_off(row, k8)) = lo;
  }
}

__global__ void __launch_bounds__(TC_THREADS, 1)
    k_rotate_tc(const Tables t, int ks_begin, float2 *__restrict__ X, const unsigned char *__restrict__ img,
                long long img_stride, int *__restrict__ status) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bars[3];
  __shared__ uint32_t tmem_slot;
  __shared__ int s_ok;
  const int ksi = ks_begin + blockIdx.y;
  const KSetDev &K = t.ks[ksi];
  if (!t.sys[K.sys].active) return;
  const int g0 = blockIdx.x * TC_M;
  if (g0 >= K.npw) return;
  const int nb = K.nb;
  const int N = ((2 * nb + 15) / 16) * 16;  // output columns
  const int KT = 2 * nb;                     // contraction length (reals)
  const int tid = threadIdx.x, warp = tid >> 5;
  const uint32_t a_bytes = TC_M * TC_KB * 2, b_bytes = (uint32_t)N * TC_KB * 2;
  const uint32_t stage_bytes = 2 * a_bytes + 2 * b_bytes;
  unsigned char *stage[2] = {smem_raw, smem_raw + stage_bytes};
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_slot)),
                 "r"(256)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_init(&bars[2], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = idesc_bf16(TC_M, N);
  float2 *Xb = X + K.psi_off;
  const unsigned char *Bimg = img + (long long)blockIdx.y * img_stride;
  const int nkb = (KT + TC_KB - 1) / TC_KB;
  bool ok = true;
  for (int kb = 0; kb < nkb; ++kb) {
    const int s = kb & 1;
    if (kb >= 2) {
      if (tid == 0) s_ok = mbar_wait(&bars[s], ((kb - 2) >> 1) & 1, g_stage_wait_limit) ? 1 : 0;
      __syncthreads();
      if (!s_ok) {
        ok = false;
        break;
      }
    }
    unsigned char *A_hi = stage[s], *A_lo = A_hi + a_bytes, *B_hi = A_lo + a_bytes,
                  *B_lo = B_hi + b_bytes;
    const int ib = kb * (TC_KB / 2);  // first band of this K block
    // B: this K block's hi and lo parts, contiguous in the image, copied as is
    {
      const unsigned char *src = Bimg + (size_t)kb * 2 * b_bytes;
      for (int i = tid; i < (int)(2 * b_bytes / 16); i += TC_THREADS) cp_async16_tc(B_hi + 16 * i, src + 16 * i);
      asm volatile("cp.async.commit_group;" ::: "memory");
    }
    // A: row g, chunk k8 holds bands ib + 4 k8 .. +3 as (re, im) pairs
    for (int c = tid; c < TC_M * 8; c += TC_THREADS) {
      const int row = c % TC_M, k8 = c / TC_M;
      const int g = g0 + row;
      float v[8];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int i = ib + 4 * k8 + q;
        float2 x = make_float2(0.f, 0.f);
        if (g < K.npw && i < nb) x = Xb[(long long)i * K.npw_pad + g];
        v[2 * q] = x.x;
        v[2 * q + 1] = x.y;
      }
      uint4 hi, lo;
      split8(v, hi, lo);
      *reinterpret_cast<uint4 *>(A_hi + core_off(row, k8)) = hi;
      *reinterpret_cast<uint4 *>(A_lo + core_off(row, k8)) = lo;
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t ah = smem_u32(A_hi), al = smem_u32(A_lo), bh = smem_u32(B_hi), bl = smem_u32(B_lo);
#pragma unroll
      for (int ks = 0; ks < TC_KB / 16; ++ks) {
        const uint32_t o = ks * 256;
        const uint64_t dah = smem_desc(ah + o, 128, 1024), dal = smem_desc(al + o, 128, 1024);
        const uint64_t dbh = smem_desc(bh + o, 128, 1024), dbl = smem_desc(bl + o, 128, 1024);
        mma_bf16(tmem, dah, dbh, idesc, (kb > 0 || ks > 0) ? 1u : 0u);
        mma_bf16(tmem, dah, dbl, idesc, 1u);
        mma_bf16(tmem, dal, dbh, idesc, 1u);
        mma_bf16(tmem, dal, dbl, idesc, 1u);
      }
      mma_commit(&bars[s]);
    }
  }
  if (tid == 0) {
    mma_commit(&bars[2]);
    s_ok = mbar_wait(&bars[2], 0) ? 1 : 0;
  }
  __syncthreads();
  if (!s_ok) ok = false;
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok) {
    const int quarter = warp & 3, half = warp >> 2;
    const int row = quarter * 32 + (tid & 31);
    const int g = g0 + row;
    const int ncol_half = N / 2;  // multiple of 8
    const int cbeg = half * ncol_half;
    for (int c = cbeg; c < cbeg + ncol_half; c += 16) {
      uint32_t r[16];
      tmem_ld16(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)c, r);
      if (g < K.npw) {
#pragma unroll
        for (int q = 0; q < 16; q += 2) {
          const int j = (c + q) >> 1;
          if (c + q < 2 * nb)
            Xb[(long long)j * K.npw_pad + g] = make_float2(__uint_as_float(r[q]), __uint_as_float(r[q + 1]));
        }
      }
    }
  } else if (tid == 0) {
    atomicExch(status + ksi, DEREK_ERR_TIMEOUT);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(256) : "memory");
  }
}

int set_stage_wait_limit(long iterations) {
  const long v = iterations < 0 ? kWaitLimit : iterations;
  return cudaMemcpyToSymbol(g_stage_wait_limit, &v, sizeof(v)) == cudaSuccess ? DEREK_OK : DEREK_ERR_CUDA;
}

void launch_rotate_tc(const Tables &t, int ks_begin, int nks, int max_nb, int max_npw, float2 *X,
                      const double2 *C, const long long *mat_off, unsigned char *img, int *status,
                      cudaStream_t st) {
  if (nks <= 0) return;
  const long long stride = (long long)rotate_tc_image_bytes(max_nb);
  derek::note_launch(), k_rotate_operand<<<dim3(4, nks), 256, 0, st>>>(t, ks_begin, C, mat_off, img, stride);
  const size_t sm = overlap_tc_smem(max_nb);
  cudaFuncSetAttribute(k_rotate_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  dim3 grid((max_npw + TC_M - 1) / TC_M, nks);
  derek::note_launch(), k_rotate_tc<<<grid, TC_THREADS, sm, st>>>(t, ks_begin, X, img, stride, status);
}

}  // namespace derek
