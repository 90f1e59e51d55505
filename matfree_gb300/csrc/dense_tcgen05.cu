// Dense operator application W = A V on the 5th-generation tensor cores.
//
//   W[b][m] = sum_k A[m][k] V[b][k] + shift * Vf[b][m]
//
// A (n x n, row-major, bf16 hi and optionally lo) and the probe panel V
// (p rows of bf16, hi and optionally lo) are both K-major, so one tile of the
// product is the UMMA D[M = 128 rows of A][N = probes] += A_tile[M][K] B[N][K]^T.
//
// CTA organisation (192 threads, one output tile of 128 rows x BN probes):
//   warp 0      TMA producer: one elected lane streams 32-wide K slices of A
//               (and A_lo) and of the panel (and its lo part) into a ring of
//               shared-memory stages (64-byte swizzled rows, 1024-byte aligned
//               tiles; 4 stages in split mode, 8 in plain bf16) and arms the
//               stage's "full" mbarrier with the transaction bytes.
//   warp 1      allocates the TMEM accumulator (BN fp32 columns x 128 lanes);
//               one lane issues tcgen05.mma (kind::f16, bf16 inputs, fp32
//               accumulate), 2 per K slice (K = 16 each), 6 for the split
//               product hi*hi + hi*lo + lo*hi, then tcgen05.commit to the
//               stage's "empty" mbarrier; a final commit signals the epilogue.
//   warps 2-5   epilogue: tcgen05.ld 32 lanes x 16 columns at a time (each
//               warp owns the TMEM lane quarter its warp index allows), add
//               shift * Vf and store; 32 lanes write 32 consecutive rows of
//               one probe (128-byte coalesced stores).
//
// Every mbarrier wait is bounded.  A role that gives up records
// MFG_ERR_TIMEOUT in *status and raises a shared abort flag; the others leave
// their loops, in-flight TMA copies and MMAs are drained with bounded waits,
// and the TMEM columns are freed before the CTA exits.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "common.cuh"
#include "kernels.cuh"

namespace mfg {

constexpr int kBM = 128;            // rows of A per tile (UMMA M)
constexpr int kBK = 32;             // K per stage: one swizzle atom row of bf16
constexpr int kRowBytes = kBK * 2;  // 64-byte rows -> SWIZZLE_64B (128 -> SWIZZLE_128B)
static_assert(kRowBytes == 64 || kRowBytes == 128, "supported swizzle widths");
constexpr int kUmmaK = 16;          // K per tcgen05.mma of kind::f16
constexpr int kGemmThreads = 192;
constexpr int64_t kPairMinRows = 1024;  // CTA pairs from this operator size on

struct GemmShared {
  uint64_t full[8];
  uint64_t empty[8];
  uint64_t tmem_full;
  uint64_t drain;
  uint32_t tmem_base;
  int abort;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// Bounded, sleeping wait; gives up early when another role raised the abort
// flag, and raises it (with MFG_ERR_TIMEOUT) when the time limit runs out.
template <bool kSleep = false>
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag,
                                          int *status) {
  if (mbar_wait_bounded<kSleep>(smem_u32(bar), parity, abort_flag)) return true;
  if (!*abort_flag) {
    *abort_flag = 1;
    if (status) atomicExch(status, (int)MFG_ERR_TIMEOUT);
  }
  return false;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int x,
                                            int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];"
      ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y)
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// UMMA shared-memory descriptor of a K-major swizzled tile whose rows are
// kRowBytes apart (the TMA box width): stride between 8-row groups (SBO) =
// 8 * kRowBytes, descriptor version 1, layout type 4 (SWIZZLE_64B) or 2
// (SWIZZLE_128B).  The leading-byte offset is not used by swizzled K-major
// layouts and is set to 1.
__device__ __forceinline__ uint64_t sw_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1u << 16;
  d |= (uint64_t)((8u * kRowBytes) >> 4) << 32;
  d |= (uint64_t)1u << 46;
  d |= (uint64_t)(kRowBytes == 128 ? 2u : 4u) << 61;
  return d;
}

// Instruction descriptor of kind::f16: D fp32, A and B bf16, both K-major.
__host__ __device__ constexpr uint32_t instr_desc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                          uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
      ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

template <bool kSplit>
__global__ void __launch_bounds__(kGemmThreads, 1)
dense_tcgen05_kernel(const __grid_constant__ CUtensorMap map_ahi,
                     const __grid_constant__ CUtensorMap map_alo,
                     const __grid_constant__ CUtensorMap map_bhi,
                     const __grid_constant__ CUtensorMap map_blo, const float *__restrict__ Vf,
                     int64_t ldvf, float *__restrict__ W, int64_t ldw, int n, int p, int BN,
                     int stages, uint32_t tmem_cols, float shift, int *status) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  // 1024-byte aligned stage ring, then the barrier block
  uint8_t *tiles = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  const uint32_t a_bytes = kBM * kBK * 2;
  const uint32_t b_bytes = (uint32_t)BN * kBK * 2;
  const uint32_t stage_bytes = (kSplit ? 2u : 1u) * (a_bytes + b_bytes);
  GemmShared *sh = reinterpret_cast<GemmShared *>(tiles + (size_t)stages * stage_bytes);

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * kBM;
  const int b0 = blockIdx.y * BN;
  const int num_k = (n + kBK - 1) / kBK;
  volatile int *abort_flag = &sh->abort;

  if (threadIdx.x == 0) {
    for (int s = 0; s < stages; ++s) {
      mbar_init(&sh->full[s], 1);
      mbar_init(&sh->empty[s], 1);
    }
    mbar_init(&sh->tmem_full, 1);
    mbar_init(&sh->drain, 1);
    sh->abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&sh->tmem_base)),
                 "r"(tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = sh->tmem_base;

  if (warp == 0) {
    if (lane == 0) {
      int issued = 0;
      for (int kt = 0; kt < num_k; ++kt) {
        const int s = kt % stages;
        const uint32_t ph = (uint32_t)(kt / stages) & 1u;
        if (!mbar_wait(&sh->empty[s], ph ^ 1u, abort_flag, status)) break;
        uint8_t *st = tiles + (size_t)s * stage_bytes;
        mbar_arrive_expect_tx(&sh->full[s], stage_bytes);
        const int kx = kt * kBK;
        tma_load_2d(st, &map_ahi, &sh->full[s], kx, m0);
        tma_load_2d(st + a_bytes, &map_bhi, &sh->full[s], kx, b0);
        if (kSplit) {
          tma_load_2d(st + a_bytes + b_bytes, &map_alo, &sh->full[s], kx, m0);
          tma_load_2d(st + 2 * a_bytes + b_bytes, &map_blo, &sh->full[s], kx, b0);
        }
        ++issued;
      }
      // drain: copies still in flight complete their stage's "full" phase
      if (*abort_flag) {
        for (int kt = (issued > stages ? issued - stages : 0); kt < issued; ++kt) {
          const int s = kt % stages;
          const uint32_t ph = (uint32_t)(kt / stages) & 1u;
          mbar_wait_bounded(smem_u32(&sh->full[s]), ph, nullptr, kMbarWaitNs / 8);
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = instr_desc_bf16(kBM, BN);
      int done = 0;
      for (int kt = 0; kt < num_k; ++kt) {
        const int s = kt % stages;
        const uint32_t ph = (uint32_t)(kt / stages) & 1u;
        if (!mbar_wait(&sh->full[s], ph, abort_flag, status)) break;
        tc_fence_after();
        const uint32_t st = smem_u32(tiles + (size_t)s * stage_bytes);
        const uint32_t ahi = st, bhi = st + a_bytes;
        const uint32_t alo = st + a_bytes + b_bytes, blo = st + 2 * a_bytes + b_bytes;
#pragma unroll
        for (int kk = 0; kk < kBK / kUmmaK; ++kk) {
          const uint32_t off = (uint32_t)kk * kUmmaK * 2;  // 32 bytes along K inside the atom
          const uint32_t acc = (kt > 0 || kk > 0) ? 1u : 0u;
          umma_bf16(tmem, sw_desc(ahi + off), sw_desc(bhi + off), idesc, acc);
          if (kSplit) {
            umma_bf16(tmem, sw_desc(ahi + off), sw_desc(blo + off), idesc, 1u);
            umma_bf16(tmem, sw_desc(alo + off), sw_desc(bhi + off), idesc, 1u);
          }
        }
        umma_commit(&sh->empty[s]);
        ++done;
      }
      // every MMA issued so far completes before this arrives
      umma_commit(done == num_k ? &sh->tmem_full : &sh->drain);
      if (done != num_k) {
        mbar_wait_bounded(smem_u32(&sh->drain), 0, nullptr, kMbarWaitNs / 8);
      }
    }
  } else {
    // epilogue: warps 2..5 -> TMEM lane quarters 2, 3, 0, 1
    const int quarter = warp & 3;
    const int row = quarter * 32 + lane;
    const int m = m0 + row;
    // The shift term's probe values (shift * V[b][m]) are loaded one group of
    // 16 probes ahead of the accumulator reads, the first group while the
    // main loop runs, so their latency stays off the epilogue's path.
    float sv[16], svn[16];
    auto load_shift = [&](int c, float(&dst)[16]) {
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int b = b0 + c + j;
        dst[j] = (shift != 0.f && m < n && b < p) ? __ldg(Vf + (int64_t)b * ldvf + m) : 0.f;
      }
    };
    load_shift(0, sv);
    // warp-uniform decision: tcgen05.ld is executed by all 32 lanes or none
    // the epilogue sleeps through the main loop
    const bool ok = __all_sync(0xffffffffu, mbar_wait<true>(&sh->tmem_full, 0, abort_flag, status));
    tc_fence_after();
    if (ok) {
      for (int c = 0; c < BN; c += 16) {
        if (c + 16 < BN) load_shift(c + 16, svn);
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)c, v);
        if (m < n) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int b = b0 + c + j;
            if (b < p) W[(int64_t)b * ldw + m] = fmaf(shift, sv[j], v[j]);
          }
        }
#pragma unroll
        for (int j = 0; j < 16; ++j) sv[j] = svn[j];
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tmem_cols)
                 : "memory");
  }
}

// ---------------------------------------------------------------------------
// 2-SM form (tcgen05 cta_group::2): a cluster of two CTAs computes one tile
// of 256 operator rows x BN probes.  Each CTA loads its own 128 rows of A
// (hi, lo) and its own half of the panel tile (BN / 2 probes, hi, lo); the
// pair's tensor cores exchange the panel halves, so every SM streams a third
// fewer bytes per flop than the one-CTA form, and the smaller stages leave
// room for a deeper ring.  All copies of a stage complete on the lead CTA's
// "full" barrier (the lead arms it with both CTAs' bytes); the lead CTA's
// MMA thread issues the M = 256 MMAs and its commits arrive on the "empty"
// and "tmem_full" barriers of both CTAs.  Each CTA's epilogue reads its own
// 128 TMEM lanes.
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

// shared::cluster address of the same shared variable in CTA `rank`
__device__ __forceinline__ uint32_t map_to_rank(uint32_t saddr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(saddr), "r"(rank));
  return r;
}

__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
  asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// 2-D tile copy into this CTA's shared memory completing on a barrier that
// may live in the peer CTA (shared::cluster address).
__device__ __forceinline__ void tma_load_2d_pair(void *dst, const CUtensorMap *map, uint32_t bar_cluster,
                                                 int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%3, %4}], [%2];"
      ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(bar_cluster), "r"(x), "r"(y)
      : "memory");
}

__device__ __forceinline__ void umma_bf16_pair(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                               uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
      ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// arrive on the barrier at the same offset in both CTAs of the pair once the
// MMAs issued so far have completed
__device__ __forceinline__ void umma_commit_pair(uint64_t *bar) {
  const uint16_t mask = 0x3;
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;"
      ::"r"(smem_u32(bar)), "h"(mask)
      : "memory");
}

// arrive on this CTA's barrier only
__device__ __forceinline__ void umma_commit_pair_local(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

template <bool kSplit>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kGemmThreads, 1)
dense_tcgen05_pair_kernel(const __grid_constant__ CUtensorMap map_ahi,
                          const __grid_constant__ CUtensorMap map_alo,
                          const __grid_constant__ CUtensorMap map_bhi,
                          const __grid_constant__ CUtensorMap map_blo, const float *__restrict__ Vf,
                          int64_t ldvf, float *__restrict__ W, int64_t ldw, int n, int p, int BN,
                          int stages, uint32_t tmem_cols, float shift, int *status) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *tiles = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  const uint32_t a_bytes = kBM * kBK * 2;                 // this CTA's 128 operator rows
  const uint32_t b_bytes = (uint32_t)(BN / 2) * kBK * 2;  // this CTA's half of the probe tile
  const uint32_t stage_bytes = (kSplit ? 2u : 1u) * (a_bytes + b_bytes);
  GemmShared *sh = reinterpret_cast<GemmShared *>(tiles + (size_t)stages * stage_bytes);

  const uint32_t rank = cluster_rank();
  const bool lead = rank == 0;
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int m0 = (int)(blockIdx.x >> 1) * (2 * kBM) + (int)rank * kBM;
  const int b0 = blockIdx.y * BN;
  const int bh = b0 + (int)rank * (BN / 2);
  // K slices of this CTA: all of them, or one half when the grid splits K
  // (gridDim.z = 2; the two partial products then add into a zeroed W)
  const int num_k_all = (n + kBK - 1) / kBK;
  const int kb0 = (int)((int64_t)num_k_all * blockIdx.z / gridDim.z);
  const int num_k = (int)((int64_t)num_k_all * (blockIdx.z + 1) / gridDim.z) - kb0;
  const bool split_k = gridDim.z > 1;
  volatile int *abort_flag = &sh->abort;

  if (threadIdx.x == 0) {
    for (int s = 0; s < stages; ++s) {
      mbar_init(&sh->full[s], 1);
      mbar_init(&sh->empty[s], 1);
    }
    mbar_init(&sh->tmem_full, 1);
    mbar_init(&sh->drain, 1);
    sh->abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    // one warp of each CTA of the pair allocates, collectively
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&sh->tmem_base)),
                 "r"(tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  // barriers of both CTAs are initialised before any copy or commit reaches them
  cluster_sync_all();
  tc_fence_after();
  const uint32_t tmem = sh->tmem_base;
  const uint32_t full0_lead = map_to_rank(smem_u32(&sh->full[0]), 0);

  if (warp == 0) {
    if (lane == 0) {
      int issued = 0;
      for (int kt = 0; kt < num_k; ++kt) {
        const int s = kt % stages;
        const uint32_t ph = (uint32_t)(kt / stages) & 1u;
        if (!mbar_wait(&sh->empty[s], ph ^ 1u, abort_flag, status)) break;
        uint8_t *st = tiles + (size_t)s * stage_bytes;
        const uint32_t full_s = full0_lead + (uint32_t)(s * sizeof(uint64_t));
        if (lead) mbar_arrive_expect_tx(&sh->full[s], 2u * stage_bytes);
        const int kx = (kb0 + kt) * kBK;
        tma_load_2d_pair(st, &map_ahi, full_s, kx, m0);
        tma_load_2d_pair(st + a_bytes, &map_bhi, full_s, kx, bh);
        if (kSplit) {
          tma_load_2d_pair(st + a_bytes + b_bytes, &map_alo, full_s, kx, m0);
          tma_load_2d_pair(st + 2 * a_bytes + b_bytes, &map_blo, full_s, kx, bh);
        }
        ++issued;
      }
      // drain (lead CTA): the copies of both CTAs complete on its "full" barriers
      if (*abort_flag && lead) {
        for (int kt = (issued > stages ? issued - stages : 0); kt < issued; ++kt) {
          const int s = kt % stages;
          const uint32_t ph = (uint32_t)(kt / stages) & 1u;
          mbar_wait_bounded(smem_u32(&sh->full[s]), ph, nullptr, kMbarWaitNs / 8);
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0 && lead) {
      const uint32_t idesc = instr_desc_bf16(2 * kBM, BN);
      int done = 0;
      for (int kt = 0; kt < num_k; ++kt) {
        const int s = kt % stages;
        const uint32_t ph = (uint32_t)(kt / stages) & 1u;
        if (!mbar_wait(&sh->full[s], ph, abort_flag, status)) break;
        tc_fence_after();
        const uint32_t st = smem_u32(tiles + (size_t)s * stage_bytes);
        const uint32_t ahi = st, bhi = st + a_bytes;
        const uint32_t alo = st + a_bytes + b_bytes, blo = st + 2 * a_bytes + b_bytes;
#pragma unroll
        for (int kk = 0; kk < kBK / kUmmaK; ++kk) {
          const uint32_t off = (uint32_t)kk * kUmmaK * 2;
          const uint32_t acc = (kt > 0 || kk > 0) ? 1u : 0u;
          umma_bf16_pair(tmem, sw_desc(ahi + off), sw_desc(bhi + off), idesc, acc);
          if (kSplit) {
            umma_bf16_pair(tmem, sw_desc(ahi + off), sw_desc(blo + off), idesc, 1u);
            umma_bf16_pair(tmem, sw_desc(alo + off), sw_desc(bhi + off), idesc, 1u);
          }
        }
        umma_commit_pair(&sh->empty[s]);
        ++done;
      }
      if (done == num_k) {
        umma_commit_pair(&sh->tmem_full);
      } else {
        umma_commit_pair_local(&sh->drain);
        mbar_wait_bounded(smem_u32(&sh->drain), 0, nullptr, kMbarWaitNs / 8);
      }
    }
  } else {
    // epilogue: warps 2..5 -> TMEM lane quarters 2, 3, 0, 1 of this CTA's rows
    const int quarter = warp & 3;
    const int m = m0 + quarter * 32 + lane;
    // The shift term's probe values (shift * V[b][m]) are loaded one group of
    // 16 probes ahead of the accumulator reads, the first group while the
    // main loop runs, so their latency stays off the epilogue's path.
    float sv[16], svn[16];
    auto load_shift = [&](int c, float(&dst)[16]) {
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int b = b0 + c + j;
        dst[j] = (shift != 0.f && blockIdx.z == 0 && m < n && b < p) ? __ldg(Vf + (int64_t)b * ldvf + m)
                                                                      : 0.f;
      }
    };
    load_shift(0, sv);
    const bool ok = __all_sync(0xffffffffu, mbar_wait<true>(&sh->tmem_full, 0, abort_flag, status));
    tc_fence_after();
    if (ok) {
      for (int c = 0; c < BN; c += 16) {
        if (c + 16 < BN) load_shift(c + 16, svn);
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)c, v);
        if (m < n) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int b = b0 + c + j;
            if (b < p) {
              const float out = fmaf(shift, sv[j], v[j]);
              // two partial products: a two-term sum is the same in either order
              if (split_k)
                atomicAdd(W + (int64_t)b * ldw + m, out);
              else
                W[(int64_t)b * ldw + m] = out;
            }
          }
        }
#pragma unroll
        for (int j = 0; j < 16; ++j) sv[j] = svn[j];
      }
    }
  }
  __syncwarp();
  tc_fence_before();
  // neither CTA releases its TMEM or shared memory while the pair's MMAs,
  // copies or commits may still reach it
  cluster_sync_all();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tmem_cols)
                 : "memory");
  }
}

// ---------------------------------------------------------------------------
// Persistent 2-SM form: one CTA pair per pair of SMs, each working through a
// fixed list of K ranges of output tiles, so that the last wave of tiles is
// spread over every SM instead of leaving some of them idle (n = 16384,
// 256 probes: 64 tiles on 76 pairs).
//
// Tiles are numbered row tile first (t = probe tile * tiles_m + row tile).
// Pair q works, in order, on
//   * the full tiles q, q + P, ..., q + (F - 1) P (the full waves), then
//   * of the R = T - F P remainder tiles, either the main K range [0, Km) of
//     tile F P + q (q < R), or the tail K range [Km, K) of the remainder
//     tiles e, e + (P - R), e + 2 (P - R), ... (e = q - R).
// Km balances the main piece against the c = ceil(R / (P - R)) tails of the
// busiest spare pair.  Tiles are split only when there are no full waves
// (F = 0), so every output row has the same accumulation structure.  A split
// tile has exactly two partial products,
// which add into a zeroed W: a two-term sum is the same in either order, so
// the result does not depend on timing.  The piece that starts at K = 0
// adds the shift term.
//
// Two TMEM accumulators (2 x BN columns) alternate between work items: the
// MMAs of item i + 1 run while the epilogue drains item i.  The epilogue
// warps of both CTAs release an accumulator by arriving on the lead CTA's
// "tmem_empty" barrier of that buffer (8 arrivals).
// ---------------------------------------------------------------------------

struct PairSchedule {
  int tiles_m;  // 256-row tiles per probe tile
  int P;        // CTA pairs of the grid
  int F;        // full waves
  int R;        // remainder tiles (main + tail pieces)
  int Km;       // K slices of a main piece; >= K: remainder tiles not split
};

// Work item i of pair q: tile and K-slice range [kb, ke); false past the end.
__host__ __device__ inline bool pair_item(const PairSchedule &sc, int K, int q, int i, int &tile,
                                          int &kb, int &ke) {
  if (i < sc.F) {
    tile = q + i * sc.P;
    kb = 0;
    ke = K;
    return true;
  }
  if (sc.R == 0) return false;
  const int j = i - sc.F;
  const int base = sc.F * sc.P;
  if (q < sc.R) {
    if (j > 0) return false;
    tile = base + q;
    kb = 0;
    ke = sc.Km < K ? sc.Km : K;
    return true;
  }
  if (sc.Km >= K) return false;
  const int r = (q - sc.R) + j * (sc.P - sc.R);
  if (r >= sc.R) return false;
  tile = base + r;
  kb = sc.Km;
  ke = K;
  return true;
}

struct GemmSharedP {
  uint64_t full[8];
  uint64_t empty[8];
  uint64_t tmem_full[2];
  uint64_t tmem_empty[2];
  uint64_t drain;
  uint32_t tmem_base;
  int abort;
};

template <bool kSplit>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kGemmThreads, 1)
dense_tcgen05_pair_persistent_kernel(const __grid_constant__ CUtensorMap map_ahi,
                                     const __grid_constant__ CUtensorMap map_alo,
                                     const __grid_constant__ CUtensorMap map_bhi,
                                     const __grid_constant__ CUtensorMap map_blo,
                                     const float *__restrict__ Vf, int64_t ldvf,
                                     float *__restrict__ W, int64_t ldw, int n, int p, int BN,
                                     int stages, uint32_t acc_cols, PairSchedule sc, float shift,
                                     int *status) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *tiles = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  const uint32_t a_bytes = kBM * kBK * 2;
  const uint32_t b_bytes = (uint32_t)(BN / 2) * kBK * 2;
  const uint32_t stage_bytes = (kSplit ? 2u : 1u) * (a_bytes + b_bytes);
  GemmSharedP *sh = reinterpret_cast<GemmSharedP *>(tiles + (size_t)stages * stage_bytes);

  const uint32_t rank = cluster_rank();
  const bool lead = rank == 0;
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int q = (int)(blockIdx.x >> 1);
  const int K = (n + kBK - 1) / kBK;
  volatile int *abort_flag = &sh->abort;

  if (threadIdx.x == 0) {
    for (int s = 0; s < stages; ++s) {
      mbar_init(&sh->full[s], 1);
      mbar_init(&sh->empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&sh->tmem_full[b], 1);
      mbar_init(&sh->tmem_empty[b], 8);  // 4 epilogue warps x 2 CTAs
    }
    mbar_init(&sh->drain, 1);
    sh->abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&sh->tmem_base)),
                 "r"(2u * acc_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  cluster_sync_all();
  tc_fence_after();
  const uint32_t tmem = sh->tmem_base;
  const uint32_t full0_lead = map_to_rank(smem_u32(&sh->full[0]), 0);

  if (warp == 0) {
    if (lane == 0) {
      int g = 0;  // K slices issued over all items: the ring position
      bool stop = false;
      int tile, kb, ke;
      for (int i = 0; !stop && pair_item(sc, K, q, i, tile, kb, ke); ++i) {
        const int rt = tile % sc.tiles_m, ct = tile / sc.tiles_m;
        const int m0 = rt * (2 * kBM) + (int)rank * kBM;
        const int bh = ct * BN + (int)rank * (BN / 2);
        for (int kt = kb; kt < ke; ++kt) {
          const int s = g % stages;
          const uint32_t ph = (uint32_t)(g / stages) & 1u;
          if (!mbar_wait(&sh->empty[s], ph ^ 1u, abort_flag, status)) {
            stop = true;
            break;
          }
          uint8_t *st = tiles + (size_t)s * stage_bytes;
          const uint32_t full_s = full0_lead + (uint32_t)(s * sizeof(uint64_t));
          if (lead) mbar_arrive_expect_tx(&sh->full[s], 2u * stage_bytes);
          const int kx = kt * kBK;
          tma_load_2d_pair(st, &map_ahi, full_s, kx, m0);
          tma_load_2d_pair(st + a_bytes, &map_bhi, full_s, kx, bh);
          if (kSplit) {
            tma_load_2d_pair(st + a_bytes + b_bytes, &map_alo, full_s, kx, m0);
            tma_load_2d_pair(st + 2 * a_bytes + b_bytes, &map_blo, full_s, kx, bh);
          }
          ++g;
        }
      }
      // drain (lead CTA): the copies of both CTAs complete on its "full" barriers
      if (*abort_flag && lead) {
        for (int t = (g > stages ? g - stages : 0); t < g; ++t) {
          const int s = t % stages;
          const uint32_t ph = (uint32_t)(t / stages) & 1u;
          mbar_wait_bounded(smem_u32(&sh->full[s]), ph, nullptr, kMbarWaitNs / 8);
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0 && lead) {
      const uint32_t idesc = instr_desc_bf16(2 * kBM, BN);
      int g = 0;
      bool stop = false;
      int tile, kb, ke;
      for (int i = 0; !stop && pair_item(sc, K, q, i, tile, kb, ke); ++i) {
        const int buf = i & 1, use = i >> 1;
        // the epilogues of both CTAs have read this accumulator's last item
        if (use > 0 && !mbar_wait(&sh->tmem_empty[buf], (uint32_t)(use - 1) & 1u, abort_flag, status)) {
          stop = true;
          break;
        }
        tc_fence_after();
        const uint32_t acc_t = tmem + (uint32_t)buf * acc_cols;
        for (int kt = kb; kt < ke; ++kt) {
          const int s = g % stages;
          const uint32_t ph = (uint32_t)(g / stages) & 1u;
          if (!mbar_wait(&sh->full[s], ph, abort_flag, status)) {
            stop = true;
            break;
          }
          tc_fence_after();
          const uint32_t st = smem_u32(tiles + (size_t)s * stage_bytes);
          const uint32_t ahi = st, bhi = st + a_bytes;
          const uint32_t alo = st + a_bytes + b_bytes, blo = st + 2 * a_bytes + b_bytes;
#pragma unroll
          for (int kk = 0; kk < kBK / kUmmaK; ++kk) {
            const uint32_t off = (uint32_t)kk * kUmmaK * 2;
            const uint32_t acc = (kt > kb || kk > 0) ? 1u : 0u;
            umma_bf16_pair(acc_t, sw_desc(ahi + off), sw_desc(bhi + off), idesc, acc);
            if (kSplit) {
              umma_bf16_pair(acc_t, sw_desc(ahi + off), sw_desc(blo + off), idesc, 1u);
              umma_bf16_pair(acc_t, sw_desc(alo + off), sw_desc(bhi + off), idesc, 1u);
            }
          }
          umma_commit_pair(&sh->empty[s]);
          ++g;
        }
        if (!stop) umma_commit_pair(&sh->tmem_full[buf]);
      }
      if (stop) {
        umma_commit_pair_local(&sh->drain);
        mbar_wait_bounded(smem_u32(&sh->drain), 0, nullptr, kMbarWaitNs / 8);
      }
    }
  } else {
    // epilogue: warps 2..5 -> TMEM lane quarters 2, 3, 0, 1 of this CTA's rows
    const int quarter = warp & 3;
    const uint32_t empty_lead0 = map_to_rank(smem_u32(&sh->tmem_empty[0]), 0);
    const uint32_t empty_lead1 = map_to_rank(smem_u32(&sh->tmem_empty[1]), 0);
    int tile, kb, ke;
    for (int i = 0; pair_item(sc, K, q, i, tile, kb, ke); ++i) {
      const int buf = i & 1, use = i >> 1;
      const int rt = tile % sc.tiles_m, ct = tile / sc.tiles_m;
      const int m = rt * (2 * kBM) + (int)rank * kBM + quarter * 32 + lane;
      const int b0 = ct * BN;
      const bool with_shift = kb == 0 && shift != 0.f;
      const bool partial = kb > 0 || ke < K;
      float sv[16], svn[16];
      auto load_shift = [&](int c, float(&dst)[16]) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int b = b0 + c + j;
          dst[j] = (with_shift && m < n && b < p) ? __ldg(Vf + (int64_t)b * ldvf + m) : 0.f;
        }
      };
      load_shift(0, sv);
      const bool ok =
          __all_sync(0xffffffffu, mbar_wait<true>(&sh->tmem_full[buf], (uint32_t)use & 1u, abort_flag, status));
      tc_fence_after();
      if (!ok) break;
      const uint32_t acc_t = tmem + (uint32_t)buf * acc_cols + ((uint32_t)(quarter * 32) << 16);
      for (int c = 0; c < BN; c += 16) {
        if (c + 16 < BN) load_shift(c + 16, svn);
        float v[16];
        tmem_ld16(acc_t + (uint32_t)c, v);
        if (m < n) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int b = b0 + c + j;
            if (b < p) {
              const float out = fmaf(shift, sv[j], v[j]);
              if (partial)
                atomicAdd(W + (int64_t)b * ldw + m, out);
              else
                W[(int64_t)b * ldw + m] = out;
            }
          }
        }
#pragma unroll
        for (int j = 0; j < 16; ++j) sv[j] = svn[j];
      }
      // this warp's reads of the accumulator are complete: release it
      tc_fence_before();
      __syncwarp();
      if (lane == 0)
        asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(buf ? empty_lead1 : empty_lead0)
                     : "memory");
    }
  }
  __syncwarp();
  tc_fence_before();
  // neither CTA releases its TMEM or shared memory while the pair's MMAs,
  // copies, commits or remote arrivals may still reach it
  cluster_sync_all();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2u * acc_cols)
                 : "memory");
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *ptr = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
  });
  return fn;
}

// 2-D bf16 map: inner extent `cols` (K), `rows` rows `ld` elements apart,
// box 64 x box_rows, 128-byte swizzle, zero fill out of bounds.
static bool make_map(CUtensorMap *map, const void *base, int64_t cols, int64_t rows, int64_t ld,
                     uint32_t box_rows) {
  auto fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  cuuint32_t box[2] = {(cuuint32_t)kBK, box_rows};
  cuuint32_t estr[2] = {1, 1};
  const CUresult r =
      fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box,
         estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
         kRowBytes == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
         CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) record_error(__FILE__, __LINE__, "cuTensorMapEncodeTiled (bf16 tile) failed");
  return r == CUDA_SUCCESS;
}

bool make_plain_tensor_map_2d(void *map128, int elem_bytes, const void *base, int64_t cols,
                              int64_t rows, int64_t ld, uint32_t box_cols, uint32_t box_rows) {
  auto fn = encode_fn();
  if (!fn || (elem_bytes != 4 && elem_bytes != 8)) return false;
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)ld * (cuuint64_t)elem_bytes};
  cuuint32_t box[2] = {box_cols, box_rows};
  cuuint32_t estr[2] = {1, 1};
  const CUresult r =
      fn(reinterpret_cast<CUtensorMap *>(map128),
         elem_bytes == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2,
         const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
         CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) record_error(__FILE__, __LINE__, "cuTensorMapEncodeTiled (basis tile) failed");
  return r == CUDA_SUCCESS;
}

bool tcgen05_supported_shape(int64_t n, int64_t p) {
  return n > 0 && p > 0 && n < (1ll << 31) && p < (1ll << 31) && encode_fn() != nullptr;
}

// ---------------------------------------------------------------------------
// Few right-hand sides (p <= 8, e.g. the one CG solve of a GP log-density):
// the product is a stream of the operator, so it runs on the CUDA cores as a
// GEMV over all SMs instead of as 128-row tensor-core tiles (n / 128 CTAs,
// too few to draw HBM bandwidth).  Warps own column segments of operator
// rows: 16-byte loads of A_hi / A_lo and of the bf16 panel, float sums of
// the same three products (hi hi + hi lo + lo hi), a fixed-order warp
// butterfly per probe.  The operator loads of the next 256 (one probe: 512)
// columns are issued before the current ones are used and bypass L1, which
// keeps the panel that every warp of the SM re-reads there.
// ---------------------------------------------------------------------------

constexpr int kGemvWarps = 8;

// 16 bytes of the operator, read once: not allocated in L1
__device__ __forceinline__ uint4 ld_stream16(const __nv_bfloat16 *p) {
  uint4 v;
  asm volatile("ld.global.nc.L1::no_allocate.v4.u32 {%0, %1, %2, %3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(p));
  return v;
}

__device__ __forceinline__ void bf16x8_to_float(const uint4 &u, float (&f)[8]) {
  const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    f[2 * i] = __uint_as_float(w[i] << 16);
    f[2 * i + 1] = __uint_as_float(w[i] & 0xFFFF0000u);
  }
}

// Each row is cut into kGemvSeg column segments, one warp each, so that a
// launch has kGemvSeg * n warp tasks: with one warp per row (n tasks against
// ~6000 resident warps) the last partial wave ran with too few loads in
// flight.  The segment sums are added in a fixed order.
constexpr int kGemvSeg = 4;
constexpr int kGemvRows = kGemvWarps / kGemvSeg;  // rows per CTA

// kDeep: loads of two iterations ahead in flight instead of one (for one
// probe, whose products are too few to cover the latency; with more probes
// the deeper ring costs occupancy).
template <int P, bool kSplit, bool kDeep>
__device__ __forceinline__ void gemv_rows(const __nv_bfloat16 *__restrict__ Ahi,
                                          const __nv_bfloat16 *__restrict__ Alo, int64_t lda,
                                          const __nv_bfloat16 *__restrict__ Vhi,
                                          const __nv_bfloat16 *__restrict__ Vlo, int64_t ldvb,
                                          const float *__restrict__ Vf, int64_t ldvf,
                                          float *__restrict__ W, int64_t ldw, int n, int p,
                                          float shift) {
  constexpr int kAhead = kDeep ? 512 : 256;
  __shared__ float part[kGemvWarps][P];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int seg = warp % kGemvSeg;
  const int64_t m = (int64_t)blockIdx.x * kGemvRows + warp / kGemvSeg;
  float acc[P];
#pragma unroll
  for (int b = 0; b < P; ++b) acc[b] = 0.f;
  if (m < n) {  // warp-uniform; every warp reaches the barrier below
    const __nv_bfloat16 *ah = Ahi + m * lda;
    const __nv_bfloat16 *al = kSplit ? Alo + m * lda : nullptr;
    const int n8 = n & ~7;
    const int seg_len = ((n8 / 8 + kGemvSeg - 1) / kGemvSeg) * 8;  // a multiple of 8 columns
    const int c0 = seg * seg_len;
    const int c1 = min(c0 + seg_len, n8);
    const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
    uint4 h0 = zero, l0 = zero, h1 = zero, l1 = zero;
    const int cl = c0 + lane * 8;
    if (cl < c1) {
      h0 = ld_stream16(ah + cl);
      if (kSplit) l0 = ld_stream16(al + cl);
    }
    if (kDeep && cl + 256 < c1) {
      h1 = ld_stream16(ah + cl + 256);
      if (kSplit) l1 = ld_stream16(al + cl + 256);
    }
    for (int c = cl; c < c1; c += 256) {
      uint4 h2 = zero, l2 = zero;
      if (c + kAhead < c1) {
        h2 = ld_stream16(ah + c + kAhead);
        if (kSplit) l2 = ld_stream16(al + c + kAhead);
      }
      float a1[8], a2[8];
      bf16x8_to_float(h0, a1);
      if (kSplit) bf16x8_to_float(l0, a2);
      if (kDeep) {
        h0 = h1;
        l0 = l1;
        h1 = h2;
        l1 = l2;
      } else {
        h0 = h2;
        l0 = l2;
      }
#pragma unroll
      for (int b = 0; b < P; ++b) {
        if (b >= p) break;
        float v1[8], v2[8];
        bf16x8_to_float(__ldg(reinterpret_cast<const uint4 *>(Vhi + b * ldvb + c)), v1);
        if (kSplit)
          bf16x8_to_float(__ldg(reinterpret_cast<const uint4 *>(Vlo + b * ldvb + c)), v2);
#pragma unroll
        for (int t = 0; t < 8; ++t) {
          acc[b] = fmaf(a1[t], v1[t], acc[b]);
          if (kSplit) {
            acc[b] = fmaf(a1[t], v2[t], acc[b]);
            acc[b] = fmaf(a2[t], v1[t], acc[b]);
          }
        }
      }
    }
    if (seg == kGemvSeg - 1) {
      for (int c = n8 + lane; c < n; c += 32) {  // columns past the last multiple of 8
        const float x1 = __bfloat162float(ah[c]);
        const float x2 = kSplit ? __bfloat162float(al[c]) : 0.f;
#pragma unroll
        for (int b = 0; b < P; ++b) {
          if (b >= p) break;
          const float y1 = __bfloat162float(Vhi[b * ldvb + c]);
          acc[b] = fmaf(x1, y1, acc[b]);
          if (kSplit) {
            acc[b] = fmaf(x1, __bfloat162float(Vlo[b * ldvb + c]), acc[b]);
            acc[b] = fmaf(x2, y1, acc[b]);
          }
        }
      }
    }
#pragma unroll
    for (int b = 0; b < P; ++b) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc[b] += __shfl_xor_sync(0xffffffffu, acc[b], o);
    }
  }
  if (lane == 0) {
#pragma unroll
    for (int b = 0; b < P; ++b) part[warp][b] = acc[b];
  }
  __syncthreads();
  if (threadIdx.x < kGemvRows * P) {
    const int r = threadIdx.x / P, b = threadIdx.x % P;
    const int64_t row = (int64_t)blockIdx.x * kGemvRows + r;
    if (row < n && b < p) {
      float t = 0.f;
#pragma unroll
      for (int q = 0; q < kGemvSeg; ++q) t += part[r * kGemvSeg + q][b];
      W[b * ldw + row] = fmaf(shift, __ldg(Vf + b * ldvf + row), t);
    }
  }
}

// one probe: 48 registers keep five CTAs on an SM with the deeper ring
template <bool kSplit>
__global__ void __launch_bounds__(32 * kGemvWarps, 5)
dense_gemv1_kernel(const __nv_bfloat16 *__restrict__ Ahi, const __nv_bfloat16 *__restrict__ Alo,
                   int64_t lda, const __nv_bfloat16 *__restrict__ Vhi,
                   const __nv_bfloat16 *__restrict__ Vlo, int64_t ldvb,
                   const float *__restrict__ Vf, int64_t ldvf, float *__restrict__ W, int64_t ldw,
                   int n, int p, float shift) {
  gemv_rows<1, kSplit, true>(Ahi, Alo, lda, Vhi, Vlo, ldvb, Vf, ldvf, W, ldw, n, p, shift);
}

template <int P, bool kSplit>
__global__ void __launch_bounds__(32 * kGemvWarps)
dense_gemv_kernel(const __nv_bfloat16 *__restrict__ Ahi, const __nv_bfloat16 *__restrict__ Alo,
                  int64_t lda, const __nv_bfloat16 *__restrict__ Vhi,
                  const __nv_bfloat16 *__restrict__ Vlo, int64_t ldvb,
                  const float *__restrict__ Vf, int64_t ldvf, float *__restrict__ W, int64_t ldw,
                  int n, int p, float shift) {
  gemv_rows<P, kSplit, false>(Ahi, Alo, lda, Vhi, Vlo, ldvb, Vf, ldvf, W, ldw, n, p, shift);
}

template <int P>
static void launch_gemv_p(bool split, const __nv_bfloat16 *A_hi, const __nv_bfloat16 *A_lo,
                          int64_t lda, const __nv_bfloat16 *V_hi, const __nv_bfloat16 *V_lo,
                          int64_t ldvb, const float *Vf, int64_t ldvf, float *W, int64_t ldw,
                          int n, int p, float shift, cudaStream_t s) {
  const unsigned grid = (unsigned)((n + kGemvRows - 1) / kGemvRows);
  if constexpr (P == 1) {
    if (split)
      dense_gemv1_kernel<true><<<grid, 32 * kGemvWarps, 0, s>>>(A_hi, A_lo, lda, V_hi, V_lo, ldvb,
                                                                Vf, ldvf, W, ldw, n, p, shift);
    else
      dense_gemv1_kernel<false><<<grid, 32 * kGemvWarps, 0, s>>>(A_hi, A_lo, lda, V_hi, V_lo,
                                                                 ldvb, Vf, ldvf, W, ldw, n, p, shift);
  } else {
    if (split)
      dense_gemv_kernel<P, true><<<grid, 32 * kGemvWarps, 0, s>>>(A_hi, A_lo, lda, V_hi, V_lo,
                                                                  ldvb, Vf, ldvf, W, ldw, n, p, shift);
    else
      dense_gemv_kernel<P, false><<<grid, 32 * kGemvWarps, 0, s>>>(A_hi, A_lo, lda, V_hi, V_lo,
                                                                   ldvb, Vf, ldvf, W, ldw, n, p, shift);
  }
}

constexpr int64_t kGemvMaxP = 8;

static int launch_dense_gemv(const __nv_bfloat16 *A_hi, const __nv_bfloat16 *A_lo, int64_t lda,
                             const __nv_bfloat16 *V_hi, const __nv_bfloat16 *V_lo, int64_t ldvb,
                             const float *Vf, int64_t ldvf, float *W, int64_t ldw, int64_t n,
                             int64_t p, double shift, cudaStream_t s) {
  const bool split = A_lo != nullptr;
  const int ni = (int)n, pi = (int)p;
  const float sh = (float)shift;
  if (p == 1)
    launch_gemv_p<1>(split, A_hi, A_lo, lda, V_hi, V_lo, ldvb, Vf, ldvf, W, ldw, ni, pi, sh, s);
  else if (p == 2)
    launch_gemv_p<2>(split, A_hi, A_lo, lda, V_hi, V_lo, ldvb, Vf, ldvf, W, ldw, ni, pi, sh, s);
  else if (p <= 4)
    launch_gemv_p<4>(split, A_hi, A_lo, lda, V_hi, V_lo, ldvb, Vf, ldvf, W, ldw, ni, pi, sh, s);
  else
    launch_gemv_p<8>(split, A_hi, A_lo, lda, V_hi, V_lo, ldvb, Vf, ldvf, W, ldw, ni, pi, sh, s);
  return MFG_LAUNCH_STATUS();
}

// ---------------------------------------------------------------------------
// Tile configuration rules (set by the autotuner through mfg_gemm_tuning_add):
// for operators of n in [n_lo, n_hi] applied to p in [p_lo, p_hi] probes, the
// CTA-pair form uses probe tiles of `bn` columns and `split` selects the
// form: 1 one tile per pair, 2 K split in two halves, 3 the persistent form
// (0: the built-in choice).  The last matching rule wins.
// ---------------------------------------------------------------------------
struct GemmRule {
  int64_t n_lo, n_hi, p_lo, p_hi;
  int bn, split;
};
static std::mutex g_rules_mu;
static GemmRule g_rules[256];
static int g_nrules = 0;

int gemm_rule_add(int64_t n_lo, int64_t n_hi, int64_t p_lo, int64_t p_hi, int bn, int split) {
  if (n_lo > n_hi || p_lo > p_hi) return MFG_ERR_BAD_ARG;
  if (bn != 0 && (bn < 64 || bn > 256 || bn % 32 != 0)) return MFG_ERR_BAD_ARG;
  if (split < 0 || split > 3) return MFG_ERR_BAD_ARG;
  std::lock_guard<std::mutex> lk(g_rules_mu);
  if (g_nrules >= 256) return MFG_ERR_SCRATCH_LIMIT;
  g_rules[g_nrules++] = GemmRule{n_lo, n_hi, p_lo, p_hi, bn, split};
  return MFG_OK;
}

int gemm_rules_clear() {
  std::lock_guard<std::mutex> lk(g_rules_mu);
  g_nrules = 0;
  return MFG_OK;
}

static GemmRule gemm_rule_for(int64_t n, int64_t p) {
  std::lock_guard<std::mutex> lk(g_rules_mu);
  for (int i = g_nrules - 1; i >= 0; --i) {
    const GemmRule &r = g_rules[i];
    if (n >= r.n_lo && n <= r.n_hi && p >= r.p_lo && p <= r.p_hi) return r;
  }
  return GemmRule{0, 0, 0, 0, 0, 0};
}

// Schedule of the persistent form for T tiles of K slices on at most
// max_pairs CTA pairs (see dense_tcgen05_pair_persistent_kernel); P = 0 when
// it does not apply.  Tails shorter than min_tail slices are not split off.
PairSchedule pair_schedule(int64_t T, int tiles_m, int max_pairs, int K, int min_tail) {
  PairSchedule sc{tiles_m, 0, 0, 0, K};
  if (T <= 0 || max_pairs < 2 || K <= 0 || T > (1 << 24)) return sc;
  int P = max_pairs;
  int F = (int)(T / P), R = (int)(T % P);
  if (F == 0 && 2 * R <= P) P = 2 * R;  // one main and one tail per tile
  int Km = K;
  // Split only when every tile is split at the same K slice (no full
  // waves): the tensor pipe's fp32 accumulation truncates, so an output's
  // rounding bias depends on the length of its accumulation chains, and
  // rows with a K split next to rows without one turn a symmetric operator
  // into a slightly non-symmetric one (n = 29368, 64 probes: 5e-5 between
  // the two kinds of rows, a 3e-4 log-determinant error under Lanczos).
  if (R > 0 && F == 0) {
    const int c = (R + (P - R) - 1) / (P - R);  // tails of the busiest spare pair
    Km = (int)(((int64_t)c * K + c) / (c + 1));
    if (Km > K) Km = K;
    if (K - Km < min_tail) Km = K;
  }
  sc.P = P;
  sc.F = F;
  sc.R = R;
  sc.Km = Km;
  return sc;
}

// K slices of the busiest pair
int64_t schedule_cost(const PairSchedule &sc, int K) {
  if (sc.P <= 0) return INT64_MAX;
  int64_t cost = (int64_t)sc.F * K;
  if (sc.R > 0) {
    if (sc.Km >= K) return cost + K;
    const int c = (sc.R + (sc.P - sc.R) - 1) / (sc.P - sc.R);
    const int64_t tail = (int64_t)c * (K - sc.Km);
    cost += sc.Km > tail ? sc.Km : tail;
  }
  return cost;
}

int launch_dense_tcgen05(const __nv_bfloat16 *A_hi, const __nv_bfloat16 *A_lo, int64_t lda,
                         const __nv_bfloat16 *V_hi, const __nv_bfloat16 *V_lo, int64_t ldvb,
                         const float *Vf, int64_t ldvf, float *W, int64_t ldw, int64_t n, int64_t p,
                         double shift, int *status, cudaStream_t s) {
  if (n <= 0 || p <= 0) return MFG_OK;
  if (!tcgen05_supported_shape(n, p)) return MFG_ERR_UNSUPPORTED;
  const bool split = (A_lo != nullptr);
  if (split && V_lo == nullptr) return MFG_ERR_BAD_ARG;
  if (lda % 8 != 0 || ldvb % 8 != 0 || ((uintptr_t)A_hi & 15) || ((uintptr_t)V_hi & 15))
    return MFG_ERR_BAD_ARG;
  if (p <= kGemvMaxP)
    return launch_dense_gemv(A_hi, A_lo, lda, V_hi, V_lo, ldvb, Vf, ldvf, W, ldw, n, p, shift, s);
  // probes per tile: a multiple of 16 in [16, 256]
  const GemmRule rule = n >= kPairMinRows ? gemm_rule_for(n, p) : GemmRule{0, 0, 0, 0, 0, 0};
  const int64_t pt = p < 256 ? p : 256;
  int BN = (int)((pt + 15) / 16 * 16);
  if (rule.bn > 0 && rule.bn < BN) BN = rule.bn;  // a narrower probe tile: more tiles per operator
  uint32_t cols = 32;
  while ((int)cols < BN) cols <<= 1;
  // CTA pairs (2-SM MMAs, M = 256) once the operator spans several pair tiles
  const bool pair = n >= kPairMinRows && BN >= 64 && BN % 32 == 0;
  const uint32_t a_bytes = kBM * kBK * 2;
  const uint32_t b_bytes = (uint32_t)(pair ? BN / 2 : BN) * kBK * 2;
  const uint32_t stage_bytes = (split ? 2u : 1u) * (a_bytes + b_bytes);
  const size_t budget = 200 * 1024;
  int stages = (int)(budget / stage_bytes);
  if (stages > 8) stages = 8;
  if (stages < 2) return MFG_ERR_UNSUPPORTED;
  const size_t smem = 1024 + (size_t)stages * stage_bytes + sizeof(GemmShared);

  CUtensorMap mahi, malo, mbhi, mblo;
  const uint32_t b_rows = (uint32_t)(pair ? BN / 2 : BN);
  if (!make_map(&mahi, A_hi, n, n, lda, kBM)) return MFG_ERR_CUDA;
  if (!make_map(&mbhi, V_hi, n, p, ldvb, b_rows)) return MFG_ERR_CUDA;
  if (split) {
    if (!make_map(&malo, A_lo, n, n, lda, kBM)) return MFG_ERR_CUDA;
    if (!make_map(&mblo, V_lo, n, p, ldvb, b_rows)) return MFG_ERR_CUDA;
  } else {
    malo = mahi;
    mblo = mbhi;
  }
  if (pair) {
    // grid.x: two CTAs per 256-row tile (the cluster dimension).  When the
    // tiles cover fewer than 60 % of the SMs (e.g. n = 8192: 64 CTAs), each
    // CTA streams its rows at a fixed rate and the SMs idle, so K is split in
    // two halves (grid.z) whose partial products add into a zeroed W.
    dim3 grid((unsigned)(2 * ((n + 2 * kBM - 1) / (2 * kBM))), (unsigned)((p + BN - 1) / BN));
    if (grid.y > 65535) return MFG_ERR_UNSUPPORTED;
    static int sms = 0;
    if (sms == 0) {
      int dev = 0;
      if (cudaGetDevice(&dev) != cudaSuccess ||
          cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        sms = 152;
    }
    const int num_k_all = (int)((n + kBK - 1) / kBK);
    const bool split_default = (int64_t)grid.x * grid.y * 5 < (int64_t)sms * 3;
    const bool split_k = rule.split == 0 ? split_default : rule.split == 2;
    // the persistent form where its schedule is shorter (or a rule asks for it)
    const int tiles_m = (int)((n + 2 * kBM - 1) / (2 * kBM));
    const PairSchedule sc = pair_schedule((int64_t)tiles_m * grid.y, tiles_m, sms / 2, num_k_all, stages);
    if (sc.P > 0 && 2 * (int64_t)sc.P > 2147483647) return MFG_ERR_UNSUPPORTED;
    const int64_t pairs_t = (int64_t)tiles_m * grid.y;
    const int64_t waves_plain = (pairs_t + sms / 2 - 1) / (sms / 2);
    const bool split_ok = split_k && num_k_all >= 4 * stages;
    const int64_t plain_cost = split_ok ? ((2 * pairs_t + sms / 2 - 1) / (sms / 2)) * ((num_k_all + 1) / 2)
                                        : waves_plain * num_k_all;
    // Filling the idle SMs also lowers the clock under the power cap (n =
    // 16384, 256 probes: 1.76 -> 1.67 GHz, no net gain), so by default only
    // schedules at least 15 % shorter take the persistent form.
    const bool persistent = sc.P > 0 && (rule.split == 3 ||
                                         (rule.split == 0 && schedule_cost(sc, num_k_all) * 100 <= plain_cost * 85));
    if (persistent) {
      if (sc.R > 0 && sc.Km < num_k_all) {
        // the split (remainder) tiles add two partial products into zeroed W
        if (grid.y == 1) {
          const int64_t r0 = (int64_t)sc.F * sc.P * 2 * kBM;
          MFG_CUDA_TRY(cudaMemset2DAsync(W + r0, (size_t)ldw * sizeof(float), 0,
                                         (size_t)(n - r0) * sizeof(float), (size_t)p, s));
        } else {
          MFG_CUDA_TRY(cudaMemset2DAsync(W, (size_t)ldw * sizeof(float), 0, (size_t)n * sizeof(float),
                                         (size_t)p, s));
        }
      }
      uint32_t acc_cols = 32;
      while ((int)acc_cols < BN) acc_cols <<= 1;
      const size_t smem_p = 1024 + (size_t)stages * stage_bytes + sizeof(GemmSharedP);
      dim3 pgrid((unsigned)(2 * sc.P), 1, 1);
      if (split) {
        MFG_CUDA_TRY(cudaFuncSetAttribute(dense_tcgen05_pair_persistent_kernel<true>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_p));
        dense_tcgen05_pair_persistent_kernel<true><<<pgrid, kGemmThreads, smem_p, s>>>(
            mahi, malo, mbhi, mblo, Vf, ldvf, W, ldw, (int)n, (int)p, BN, stages, acc_cols, sc,
            (float)shift, status);
      } else {
        MFG_CUDA_TRY(cudaFuncSetAttribute(dense_tcgen05_pair_persistent_kernel<false>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_p));
        dense_tcgen05_pair_persistent_kernel<false><<<pgrid, kGemmThreads, smem_p, s>>>(
            mahi, malo, mbhi, mblo, Vf, ldvf, W, ldw, (int)n, (int)p, BN, stages, acc_cols, sc,
            (float)shift, status);
      }
      return MFG_LAUNCH_STATUS();
    }
    if (split_ok) {
      grid.z = 2;
      MFG_CUDA_TRY(cudaMemset2DAsync(W, (size_t)ldw * sizeof(float), 0, (size_t)n * sizeof(float),
                                     (size_t)p, s));
    }
    if (split) {
      MFG_CUDA_TRY(cudaFuncSetAttribute(dense_tcgen05_pair_kernel<true>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      dense_tcgen05_pair_kernel<true><<<grid, kGemmThreads, smem, s>>>(
          mahi, malo, mbhi, mblo, Vf, ldvf, W, ldw, (int)n, (int)p, BN, stages, cols,
          (float)shift, status);
    } else {
      MFG_CUDA_TRY(cudaFuncSetAttribute(dense_tcgen05_pair_kernel<false>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      dense_tcgen05_pair_kernel<false><<<grid, kGemmThreads, smem, s>>>(
          mahi, malo, mbhi, mblo, Vf, ldvf, W, ldw, (int)n, (int)p, BN, stages, cols,
          (float)shift, status);
    }
    return MFG_LAUNCH_STATUS();
  }
  dim3 grid((unsigned)((n + kBM - 1) / kBM), (unsigned)((p + BN - 1) / BN));
  if (grid.y > 65535) return MFG_ERR_UNSUPPORTED;
  if (split) {
    MFG_CUDA_TRY(cudaFuncSetAttribute(dense_tcgen05_kernel<true>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dense_tcgen05_kernel<true><<<grid, kGemmThreads, smem, s>>>(
        mahi, malo, mbhi, mblo, Vf, ldvf, W, ldw, (int)n, (int)p, BN, stages, cols, (float)shift,
        status);
  } else {
    MFG_CUDA_TRY(cudaFuncSetAttribute(dense_tcgen05_kernel<false>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dense_tcgen05_kernel<false><<<grid, kGemmThreads, smem, s>>>(
        mahi, malo, mbhi, mblo, Vf, ldvf, W, ldw, (int)n, (int)p, BN, stages, cols, (float)shift,
        status);
  }
  return MFG_LAUNCH_STATUS();
}

}  // namespace mfg

extern "C" {

// Work list of the persistent CTA-pair form (host only; see the header).
MFG_API int64_t mfg_gemm_pair_schedule(int64_t n, int64_t p, int32_t bn, int32_t max_pairs,
                                       int32_t min_tail, int32_t *items, int64_t capacity) {
  using namespace mfg;
  if (n <= 0 || p <= 0 || bn < 16 || bn > 256 || bn % 16 != 0 || max_pairs < 2 || min_tail < 0)
    return -(int64_t)MFG_ERR_BAD_ARG;
  if (n >= (1ll << 31) || p >= (1ll << 31)) return -(int64_t)MFG_ERR_BAD_ARG;
  const int K = (int)((n + kBK - 1) / kBK);
  const int tiles_m = (int)((n + 2 * kBM - 1) / (2 * kBM));
  const int64_t T = (int64_t)tiles_m * ((p + bn - 1) / bn);
  const PairSchedule sc = pair_schedule(T, tiles_m, max_pairs, K, min_tail);
  if (sc.P <= 0) return -(int64_t)MFG_ERR_UNSUPPORTED;
  int64_t count = 0;
  for (int q = 0; q < sc.P; ++q) {
    int tile, kb, ke;
    for (int i = 0; pair_item(sc, K, q, i, tile, kb, ke); ++i, ++count) {
      if (items && count < capacity) {
        items[4 * count] = q;
        items[4 * count + 1] = tile;
        items[4 * count + 2] = kb;
        items[4 * count + 3] = ke;
      }
    }
  }
  return count;
}

}  // extern "C"
