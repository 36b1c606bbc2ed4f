// emulator.cu -- radiation emulator: an MLP trained and run on the GPU with hand-written
// BF16 tensor-core kernels (tcgen05.mma, accumulators in tensor memory).
//
// GEMM kernel (persistent, one CTA per SM): C = A * B^T (A: M x K, B: N x K, both K-major
// BF16) in tiles of 128 x BN.  The K blocks of 64 reach shared memory by TMA
// (cp.async.bulk.tensor, 128-byte swizzle: 8-row x 128-byte atoms, 16-byte chunks XOR-ed by
// the row), issued by a producer warp into a ring of stages; an MMA warp waits for a stage to
// fill, issues four tcgen05.mma (M=128, N=BN, K=16, kind::f16 with BF16 inputs and an FP32
// accumulator in tensor memory; the K=16 steps advance the descriptors 32 bytes inside the
// swizzle atom) and commits them to the stage's "empty" mbarrier, which releases it to the
// producer.  Two accumulators alternate between tiles: four epilogue warps read a finished one
// with tcgen05.ld (warp w owns tensor-memory lanes 32*(w%4).. = tile rows) and apply one of the
// fused epilogues (bias + GELU with BF16 and transposed BF16 copies, bias only, GELU derivative
// for the backward pass, or plain FP32 partial sums for split-K) while the next tile's MMAs run.
// Launched with programmatic stream serialisation, so a GEMM's set-up overlaps the previous
// kernel's tail.
//
// Every wait on an mbarrier is bounded; on time-out the kernel records an error code, waits
// (bounded) once more for its own tensor-core work, frees its tensor memory and returns.
#include "lgame_emulator.h"
#include "common.h"
#include "emulator.cuh"

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

namespace emu {

typedef __nv_bfloat16 bf16;

// ---- tcgen05 / mbarrier primitives (inline PTX) ---------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor of a K-major tile of 8-row x 128-byte atoms with the
// 128-byte swizzle: start address >> 4, stride 1024 bytes between 8-row groups (bits 32-45),
// fixed version bits 46-48 = 0b001, layout type 2 at bits 61-63; the leading offset (bits
// 16-29) is not used when a row of the tile is one atom wide
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024u >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}
// one box of a 2-D tensor map (inner coordinate c0, outer c1) into shared memory, completing
// on the mbarrier's transaction count
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int c0, int c1, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(map), "r"(c0), "r"(c1), "r"(mbar)
      : "memory");
}
// instruction descriptor, kind::f16: D = F32 (bits 4-5 = 1), A = B = BF16 (bits 7-9, 10-12 = 1),
// both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28
__host__ __device__ constexpr uint32_t instr_desc(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}
__device__ __forceinline__ void tc_alloc(uint32_t dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tc_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accum) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accum)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// bounded wait for the completion of phase `parity`; false on time-out
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
  for (int it = 0; it < (1 << 22); ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
    if (it > 64) __nanosleep(64);
  }
  return false;
}
// 16 consecutive FP32 accumulator columns of this thread's lane
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
      "[%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678f)); }
__device__ __forceinline__ float gelu_grad(float z) {
  return 0.5f * (1.f + erff(z * 0.70710678f)) + z * 0.39894228f * __expf(-0.5f * z * z);
}

// ---- the GEMM -------------------------------------------------------------------------------
// Persistent: one CTA per SM loops over the output tiles (tile t, t + gridDim.x, ...), with the
// warps specialised:
//   warp 0 (lane 0)  TMA producer: the K blocks of every tile of the CTA into a ring of stages,
//                    running ahead across tile boundaries;
//   warp 1 (lane 0)  MMA issuer: four tcgen05.mma per K block into one of two accumulators in
//                    tensor memory, alternating per tile; the stage is released by a commit to its
//                    "empty" barrier, the finished accumulator by a commit to its "full" barrier;
//   warps 2-5        epilogue: warp w reads tensor-memory lanes 32*(w%4).. (tile rows) of the
//                    finished accumulator, applies the fused epilogue, and arrives on the
//                    accumulator's "empty" barrier, so that the MMAs of the next tile run while
//                    the previous one drains.
// Every wait is bounded and also ends when another role has given up (a shared abort flag);
// the CTA then waits (bounded) for its own copies and MMAs before freeing tensor memory.
constexpr int kGemmThreads = 192;

template <int BN>
struct GemmCfg {
  static constexpr uint32_t kCols = (BN <= 32) ? 32 : (BN <= 64) ? 64 : (BN <= 128) ? 128 : 256;  // one accumulator
  static constexpr uint32_t kA = 128 * 64 * 2, kB = BN * 64 * 2, kStage = kA + kB;             // bytes per stage
  static constexpr int kStages = (BN <= 128) ? 6 : 4;
  // per epilogue warp a 32 x 32 FP32 staging tile (4 KB, 128-byte swizzle) for the TMA store
  static constexpr uint32_t kStg = 32 * 32 * 4;
  static constexpr size_t kSmem = (size_t)kStages * kStage + 4 * kStg + 1024;  // + alignment slack of the atoms
};

// TMA tensor store of a 3-D box from shared memory (bulk group), and its completion waits
__device__ __forceinline__ void tma_store_3d(const CUtensorMap* map, uint32_t src, int c0, int c1, int c2) {
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%1, %2, %3}], [%4];" ::"l"(map), "r"(c0),
               "r"(c1), "r"(c2), "r"(src)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read0() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait0() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint32_t mbar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(done)
      : "r"(mbar), "r"(parity)
      : "memory");
  return done != 0;
}
// bounded wait that also gives up once *abort is set
__device__ __forceinline__ bool mbar_wait_or_abort(uint32_t mbar, uint32_t parity, const volatile int* abort) {
  for (int it = 0; it < (1 << 22); ++it) {
    if (mbar_test(mbar, parity)) return true;
    if (it > 64) {
      if (*abort) return false;
      __nanosleep(64);
    }
  }
  return false;
}

// the fused epilogue of 16 accumulator columns (nb..nb+15) of tile row m: the FP32 output
// values into f (stored by the caller), the BF16 outputs written here
__device__ __forceinline__ void epilogue16(const Epi& ep, int m, int nb, const float* v, float* f) {
  switch (ep.kind) {
    case kEpiF32:
#pragma unroll
      for (int j = 0; j < 16; ++j) f[j] = v[j];
      break;
    case kEpiBias:
#pragma unroll
      for (int j = 0; j < 16; ++j) f[j] = v[j] + ep.bias[nb + j];
      break;
    case kEpiBiasGeluH: {
      __align__(16) bf16 hb[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) hb[j] = __float2bfloat16_rn(gelu(v[j] + ep.bias[nb + j]));
      uint4* ho = reinterpret_cast<uint4*>(ep.h + (size_t)m * ep.ldh + nb);
      ho[0] = reinterpret_cast<const uint4*>(hb)[0];
      ho[1] = reinterpret_cast<const uint4*>(hb)[1];
      break;
    }
    case kEpiBiasGelu:
    case kEpiGeluBwd: {
      if (ep.kind == kEpiBiasGelu) {
#pragma unroll
        for (int j = 0; j < 16; ++j) f[j] = v[j] + ep.bias[nb + j];
      } else {
        const float4* zp = reinterpret_cast<const float4*>(ep.zprev + (size_t)m * ep.ldc + nb);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float4 t = zp[q];
          f[4 * q] = v[4 * q] * gelu_grad(t.x);
          f[4 * q + 1] = v[4 * q + 1] * gelu_grad(t.y);
          f[4 * q + 2] = v[4 * q + 2] * gelu_grad(t.z);
          f[4 * q + 3] = v[4 * q + 3] * gelu_grad(t.w);
        }
      }
      __align__(16) bf16 hb[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) hb[j] = __float2bfloat16_rn(ep.kind == kEpiBiasGelu ? gelu(f[j]) : f[j]);
      uint4* ho = reinterpret_cast<uint4*>(ep.h + (size_t)m * ep.ldh + nb);
      ho[0] = reinterpret_cast<const uint4*>(hb)[0];
      ho[1] = reinterpret_cast<const uint4*>(hb)[1];
      // the transposed BF16 copy element-wise, coalesced across the warp's rows
#pragma unroll
      for (int j = 0; j < 16; ++j) ep.ht[(size_t)(nb + j) * ep.ldt + m] = hb[j];
      break;
    }
    default: break;
  }
}

template <int BN>
__global__ void __launch_bounds__(kGemmThreads, 1) k_gemm(const __grid_constant__ CUtensorMap tmA,
                                                          const __grid_constant__ CUtensorMap tmB,
                                                          const __grid_constant__ CUtensorMap tmC, int K, int kchunk,
                                                          int tiles_n, int tiles_m, int splits, Epi ep, int* err) {
  using Cfg = GemmCfg<BN>;
  constexpr int S = Cfg::kStages;
  constexpr uint32_t kCols = Cfg::kCols, kA = Cfg::kA, kStage = Cfg::kStage;
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full[S], empty[S], acc_full[2], acc_empty[2], done;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  const volatile int* abort_v = &abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ntiles = tiles_n * tiles_m * splits;
  const uint32_t sbase = (smem_u32(smem_raw) + 1023u) & ~1023u;  // swizzle atoms are 1024-byte aligned
  // launched with programmatic stream serialisation: the next kernel of the stream may be
  // scheduled now (it waits for this grid's completion before touching memory), and this
  // grid's set-up below overlaps the previous kernel's tail until griddepcontrol.wait
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  if (tid == 0) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(&tmA) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(&tmB) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(&tmC) : "memory");
  }
  if (warp == 0) tc_alloc(smem_u32(&tmem_base), 2 * kCols);
  if (tid == 0) {
    for (int i = 0; i < S; ++i) {
      mbar_init(smem_u32(&full[i]), 1);
      mbar_init(smem_u32(&empty[i]), 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(smem_u32(&acc_full[i]), 1);
      mbar_init(smem_u32(&acc_empty[i]), 4);  // one arrival per epilogue warp
    }
    mbar_init(smem_u32(&done), 1);
    abort_flag = 0;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  // the previous kernel's results (A, B, bias, the epilogue's inputs) are complete and visible,
  // and its reads of what this grid writes are done
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const uint32_t tmem = tmem_base;
  // tile t: n tile fastest, so the CTAs that run at the same time share an A tile through L2
  auto tile_of = [&](int t, int* tn, int* tm, int* z) {
    *tn = t % tiles_n;
    const int r = t / tiles_n;
    *tm = r % tiles_m;
    *z = r / tiles_m;
  };
  auto nk_of = [&](int z) { const int k0 = z * kchunk; return (min(K, k0 + kchunk) - k0) / 64; };
  bool failed = false;
  if (warp == 0) {
    if (lane == 0) {
      int it = 0;  // K blocks issued, over all tiles
      for (int t = blockIdx.x; t < ntiles && !failed; t += gridDim.x) {
        int tn, tm, z;
        tile_of(t, &tn, &tm, &z);
        const int nk = nk_of(z), k0 = z * kchunk;
        for (int kb = 0; kb < nk; ++kb, ++it) {
          const int st = it % S;
          if (it >= S && !mbar_wait_or_abort(smem_u32(&empty[st]), (uint32_t)((it / S - 1) & 1), abort_v)) {
            failed = true;
            break;
          }
          const uint32_t a = sbase + st * kStage;
          mbar_arrive_expect_tx(smem_u32(&full[st]), kStage);
          tma_load_2d(a, &tmA, k0 + 64 * kb, tm * 128, smem_u32(&full[st]));
          tma_load_2d(a + kA, &tmB, k0 + 64 * kb, tn * BN, smem_u32(&full[st]));
        }
      }
      if (failed) {
        abort_flag = 1;
        // the copies still in flight land before the CTA exits (bounded)
        for (int j = max(0, it - S); j < it; ++j) mbar_wait(smem_u32(&full[j % S]), (uint32_t)((j / S) & 1));
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = instr_desc(128, BN);
      int it = 0, lt = 0;  // K blocks consumed, tiles of this CTA
      for (int t = blockIdx.x; t < ntiles && !failed; t += gridDim.x, ++lt) {
        int tn, tm, z;
        tile_of(t, &tn, &tm, &z);
        const int nk = nk_of(z), b = lt & 1;
        // the accumulator's previous tile (lt - 2) must have been read out
        if (lt >= 2 && !mbar_wait_or_abort(smem_u32(&acc_empty[b]), (uint32_t)((lt / 2 - 1) & 1), abort_v)) {
          failed = true;
          break;
        }
        tc_fence_after();
        const uint32_t acc = tmem + (uint32_t)b * kCols;
        for (int kb = 0; kb < nk; ++kb, ++it) {
          const int st = it % S;
          if (!mbar_wait_or_abort(smem_u32(&full[st]), (uint32_t)((it / S) & 1), abort_v)) {
            failed = true;
            break;
          }
          tc_fence_after();
          const uint32_t a = sbase + st * kStage;
#pragma unroll
          for (int s = 0; s < 4; ++s)
            tc_mma(acc, smem_desc_sw128(a + s * 32), smem_desc_sw128(a + kA + s * 32), idesc,
                   (kb > 0 || s > 0) ? 1u : 0u);
          tc_commit(smem_u32(&empty[st]));
        }
        if (failed) break;
        tc_commit(smem_u32(&acc_full[b]));
      }
      if (failed) abort_flag = 1;
      // arrives once every tensor-core operation issued above has completed (also after a failure)
      tc_commit(smem_u32(&done));
    }
  } else {
    const int qw = warp & 3;  // tensor-memory lanes 32*qw.. = tile rows
    // this warp's staging tile, after the stages (1024-byte aligned: 128-byte swizzle atoms)
    const uint32_t stg = sbase + (uint32_t)S * kStage + (uint32_t)qw * Cfg::kStg;
    uint8_t* stg_ptr = smem_raw + (stg - smem_u32(smem_raw));
    int lt = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++lt) {
      int tn, tm, z;
      tile_of(t, &tn, &tm, &z);
      const int b = lt & 1;
      bool ok = mbar_wait_or_abort(smem_u32(&acc_full[b]), (uint32_t)((lt / 2) & 1), abort_v);
      ok = __all_sync(0xffffffffu, ok);  // the tensor-memory loads below need the whole warp
      if (!ok) {
        failed = true;
        break;
      }
      tc_fence_after();
      const int m0 = tm * 128 + qw * 32, m = m0 + lane;
      for (int c = 0; c < BN; c += 32) {
        float v[32], f[32];
        const uint32_t ta = tmem + (uint32_t)b * kCols + ((uint32_t)(qw * 32) << 16) + (uint32_t)c;
        tc_ld16(ta, v);
        tc_ld16(ta + 16, v + 16);
        const int nb = tn * BN + c;
        epilogue16(ep, m, nb, v, f);
        epilogue16(ep, m, nb + 16, v + 16, f + 16);
        if (ep.kind == kEpiBiasGeluH) continue;  // no FP32 output
        // the FP32 values through the staging tile: row `lane` in the 128-byte swizzle (its
        // 16-byte chunk j at position j ^ (row % 8), so the warp's stores hit distinct banks),
        // then one TMA store of the 32 x 32 box; the previous box's read of the tile first
        if (lane == 0) bulk_wait_read0();
        __syncwarp();
        float4* row = reinterpret_cast<float4*>(stg_ptr + lane * 128);
#pragma unroll
        for (int j = 0; j < 8; ++j) row[j ^ (lane & 7)] = make_float4(f[4 * j], f[4 * j + 1], f[4 * j + 2], f[4 * j + 3]);
        fence_async_smem();
        __syncwarp();
        if (lane == 0) {
          tma_store_3d(&tmC, stg, nb, m0, ep.kind == kEpiF32 ? z : 0);
          bulk_commit();
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(&acc_empty[b]));
    }
    if (failed && lane == 0) abort_flag = 1;
    if (lane == 0) bulk_wait0();  // the tensor stores complete before the CTA exits
  }
  __syncwarp();
  const bool ok = mbar_wait(smem_u32(&done), 0);
  tc_fence_after();
  if (__syncthreads_or(failed || !ok) && tid == 0) atomicExch(err, 1);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tc_dealloc(tmem, 2 * kCols);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link to the driver library)
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  }
  return fn;
}
// encoded tensor maps, kept by their parameters: the training and inference loops use the same
// few buffers again and again, and encoding costs host time on every launch otherwise
struct MapKey {
  const void* base;
  int dtype, rank;
  cuuint64_t dims[3], strides[2];
  cuuint32_t box[3];
  bool operator==(const MapKey& o) const { return std::memcmp(this, &o, sizeof(MapKey)) == 0; }
};
int encode_cached(CUtensorMap* map, const MapKey& k) {
  static std::mutex mu;
  static std::vector<std::pair<MapKey, CUtensorMap>> cache;
  std::lock_guard<std::mutex> lock(mu);
  for (const auto& e : cache)
    if (e.first == k) { *map = e.second; return LGAME_OK; }
  const EncodeTiledFn enc = encode_tiled();
  if (!enc) return LGAME_ERR_CUDA;
  const cuuint32_t estride[3] = {1u, 1u, 1u};
  const CUresult r = enc(map, (CUtensorMapDataType)k.dtype, (cuuint32_t)k.rank, (void*)k.base, k.dims, k.strides, k.box,
                         estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return LGAME_ERR_INVALID_ARG;
  if (cache.size() >= 256) cache.erase(cache.begin());
  cache.emplace_back(k, *map);
  return LGAME_OK;
}
// tensor map of a K-major BF16 matrix (rows x K, leading dimension ld elements) in boxes of
// 64 (K) x box_rows with the 128-byte swizzle; the encoder rejects unaligned bases and strides
int tensor_map(CUtensorMap* map, const bf16* base, int rows, int K, int ld, int box_rows) {
  MapKey k{};
  k.base = base;
  k.dtype = CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
  k.rank = 2;
  k.dims[0] = (cuuint64_t)K; k.dims[1] = (cuuint64_t)rows;
  k.strides[0] = (cuuint64_t)ld * sizeof(bf16);
  k.box[0] = 64u; k.box[1] = (cuuint32_t)box_rows;
  return encode_cached(map, k);
}
// tensor map of the FP32 output: columns x rows x splits (leading dimension ldc elements, split
// stride elements) in 32 x 32 x 1 boxes with the 128-byte swizzle (the epilogue's staging tile)
int tensor_map_c(CUtensorMap* map, const float* base, int cols, int rows, int splits, int ldc, long long split_stride) {
  MapKey k{};
  k.base = base;
  k.dtype = CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
  k.rank = 3;
  k.dims[0] = (cuuint64_t)cols; k.dims[1] = (cuuint64_t)rows; k.dims[2] = (cuuint64_t)splits;
  k.strides[0] = (cuuint64_t)ldc * sizeof(float);
  k.strides[1] = (cuuint64_t)(splits > 1 ? split_stride : (long long)ldc * rows) * sizeof(float);
  k.box[0] = 32u; k.box[1] = 32u; k.box[2] = 1u;
  return encode_cached(map, k);
}

template <int BN>
int launch_gemm_bn(const bf16* A, int lda, const bf16* B, int ldb, int M, int N, int K, int splits, const Epi& ep,
                   int* err, cudaStream_t st) {
  const size_t shm = GemmCfg<BN>::kSmem;
  static bool attr_set = false;
  static int nsm = 0;
  if (!attr_set) {
    if (cudaFuncSetAttribute(k_gemm<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm) != cudaSuccess)
      return LGAME_ERR_CUDA;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      return LGAME_ERR_CUDA;
    attr_set = true;
  }
  CUtensorMap ma, mb, mc;
  const int kchunk = ((K / splits + 63) / 64) * 64;
  const int zs = (K + kchunk - 1) / kchunk;
  int rc = tensor_map(&ma, A, M, K, lda, 128);
  if (rc == LGAME_OK) rc = tensor_map(&mb, B, N, K, ldb, BN);
  if (rc == LGAME_OK) {
    if (ep.kind == kEpiBiasGeluH) mc = ma;  // no FP32 output; the map is not used
    else rc = tensor_map_c(&mc, ep.c, N, M, ep.kind == kEpiF32 ? zs : 1, ep.ldc, ep.split_stride);
  }
  if (rc != LGAME_OK) return rc;
  const int tiles_n = N / BN, tiles_m = M / 128;
  const long long ntiles = (long long)tiles_n * tiles_m * zs;
  const int grid = (int)std::min<long long>(ntiles, nsm);
  // programmatic dependent launch: see griddepcontrol in k_gemm
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(kGemmThreads);
  cfg.dynamicSmemBytes = shm;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (cudaLaunchKernelEx(&cfg, k_gemm<BN>, ma, mb, mc, K, kchunk, tiles_n, tiles_m, zs, ep, err) != cudaSuccess)
    return LGAME_ERR_CUDA;
  return cudaGetLastError() == cudaSuccess ? LGAME_OK : LGAME_ERR_CUDA;
}

int launch_gemm(const bf16* A, int lda, const bf16* B, int ldb, int M, int N, int K, int splits, const Epi& ep,
                int* err, cudaStream_t st) {
  if (M % 128 || K % 64 || N % 64 || splits < 1) return LGAME_ERR_INVALID_ARG;
  // the widest tile that still gives about two thirds of the SMs a tile (wider tiles issue
  // fuller MMAs and move fewer operand bytes from L2), else the narrowest
  const long long tiles_m = (long long)(M / 128) * splits;
  const int cand[4] = {256, 192, 128, 64};
  int bn = 0;
  for (int c : cand)
    if (N % c == 0 && tiles_m * (N / c) >= 100) { bn = c; break; }
  if (!bn)
    for (int c : {64, 128, 192, 256})
      if (N % c == 0) { bn = c; break; }
  switch (bn) {
    case 256: return launch_gemm_bn<256>(A, lda, B, ldb, M, N, K, splits, ep, err, st);
    case 192: return launch_gemm_bn<192>(A, lda, B, ldb, M, N, K, splits, ep, err, st);
    case 128: return launch_gemm_bn<128>(A, lda, B, ldb, M, N, K, splits, ep, err, st);
    default: return launch_gemm_bn<64>(A, lda, B, ldb, M, N, K, splits, ep, err, st);
  }
}

// ---- element-wise and reduction kernels ------------------------------------------------------
// Kernels that write a matrix and its transpose work on 32 x 32 tiles (blocks of 32 x 8
// threads): a warp reads and writes a row of the tile, and the transposed copy goes out
// through shared memory, so that both sides are coalesced.
//
// standardised, zero-padded BF16 inputs, row-major and transposed; grid (nin_pad/32, batch/32);
// rows >= valid (padding of the last batch) are zero and not read
__global__ void __launch_bounds__(256) k_prep_x(const float* __restrict__ x, int nin, int nin_pad, int batch,
                                                int valid, const float* mean, const float* istd, bf16* X, bf16* XT) {
  __shared__ bf16 t[32][34];
  const int c = blockIdx.x * 32 + threadIdx.x, r0 = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += 8) {
    const int r = r0 + j;
    const float v = (c < nin && r < valid) ? (x[(size_t)r * nin + c] - mean[c]) * istd[c] : 0.f;
    const bf16 b = __float2bfloat16_rn(v);
    X[(size_t)r * nin_pad + c] = b;
    t[j][threadIdx.x] = b;
  }
  if (!XT) return;  // inference: no transposed copy (only the backward pass reads it)
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += 8)
    XT[(size_t)(blockIdx.x * 32 + j) * batch + r0 + threadIdx.x] = t[threadIdx.x][j];
}
__global__ void k_prep_y(const float* __restrict__ y, int nout, int nout_pad, int batch, const float* mean,
                         const float* istd, float* Yt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= batch * nout_pad) return;
  const int r = i / nout_pad, c = i % nout_pad;
  Yt[i] = (c < nout) ? (y[(size_t)r * nout + c] - mean[c]) * istd[c] : 0.f;
}
// loss partial sums per tile and the output gradient dL/dY = 2 (Y - Yt) / (batch * nout),
// in FP32, BF16 and transposed BF16; grid (nout_pad/32, batch/32), one partial per block
__global__ void __launch_bounds__(256) k_loss_dy(const float* Y, const float* Yt, int nout, int nout_pad, int batch,
                                                 float* d32, bf16* db, bf16* dbt, float* part) {
  __shared__ bf16 t[32][34];
  __shared__ float sh[256];
  const int c = blockIdx.x * 32 + threadIdx.x, r0 = blockIdx.y * 32;
  const float scale = 2.f / (float)((double)batch * nout);
  float l = 0.f;
  for (int j = threadIdx.y; j < 32; j += 8) {
    const size_t i = (size_t)(r0 + j) * nout_pad + c;
    float d = 0.f;
    if (c < nout) {
      const float e = Y[i] - Yt[i];
      l += e * e;
      d = e * scale;
    }
    d32[i] = d;
    const bf16 b = __float2bfloat16_rn(d);
    db[i] = b;
    t[j][threadIdx.x] = b;
  }
  const int tid = threadIdx.y * 32 + threadIdx.x;
  sh[tid] = l;
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += 8)
    dbt[(size_t)(blockIdx.x * 32 + j) * batch + r0 + threadIdx.x] = t[threadIdx.x][j];
  for (int w = 128; w > 0; w >>= 1) {
    if (tid < w) sh[tid] += sh[tid + w];
    __syncthreads();
  }
  if (tid == 0) part[blockIdx.y * gridDim.x + blockIdx.x] = sh[0];
}
// deterministic column sums of a rows x cols matrix in two passes: partial sums of 32
// columns over one chunk of rows per block (grid (cols/32, chunks), warps read rows), then
// the chunks' partials summed in order
__global__ void __launch_bounds__(256) k_colsum_part(const float* a, int rows, int cols, float* part) {
  __shared__ float sh[8][33];
  const int c = blockIdx.x * 32 + threadIdx.x;
  const int per = rows / gridDim.y, r0 = blockIdx.y * per;
  float s = 0.f;
  for (int r = r0 + threadIdx.y; r < r0 + per; r += 8) s += a[(size_t)r * cols + c];
  sh[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y == 0) {
    float t = sh[0][threadIdx.x];
    for (int k = 1; k < 8; ++k) t += sh[k][threadIdx.x];
    part[(size_t)blockIdx.y * cols + c] = t;
  }
}
__global__ void k_colsum_fin(const float* part, int chunks, int cols, float* out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  float s = 0.f;
  for (int k = 0; k < chunks; ++k) s += part[(size_t)k * cols + c];
  out[c] = s;
}
// split-K partials of dW^T (in x out) summed and written transposed as dW (out x in)
__global__ void k_splitk_reduce_t(const float* part, int splits, int rows_in, int cols_out, float* gw) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows_in * cols_out) return;
  const int r = i / cols_out, c = i % cols_out;
  float s = 0.f;
  for (int z = 0; z < splits; ++z) s += part[(size_t)z * rows_in * cols_out + i];
  gw[(size_t)c * rows_in + r] = s;
}
__global__ void k_splitk_reduce(const float* part, int splits, long long n, float* out) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  float s = 0.f;
  for (int z = 0; z < splits; ++z) s += part[(size_t)z * n + i];
  out[i] = s;
}
// Adam update of one parameter matrix (rows x cols) and its BF16 copies (row-major, transposed)
__global__ void k_adam(float* p, const float* g, float* m, float* v, long long n, int cols, float lr, float b1, float b2,
                       float c1, float c2, float eps, bf16* pb, bf16* pbt, int rows) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float pi = p[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
  p[i] = pi;
  if (pb) {
    const bf16 b = __float2bfloat16_rn(pi);
    pb[i] = b;
    const long long r = i / cols, c = i % cols;
    pbt[(size_t)c * rows + r] = b;
  }
}
__global__ void k_to_bf16_t(const float* p, long long n, int cols, int rows, bf16* pb, bf16* pbt) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const bf16 b = __float2bfloat16_rn(p[i]);
  pb[i] = b;
  const long long r = i / cols, c = i % cols;
  pbt[(size_t)c * rows + r] = b;
}
__global__ void k_denorm(const float* Y, int nout, int nout_pad, int batch, const float* mean, const float* std_,
                         float* y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= batch * nout) return;
  const int r = i / nout, c = i % nout;
  y[i] = Y[(size_t)r * nout_pad + c] * std_[c] + mean[c];
}
__global__ void k_gather_rows(const float* src, const long long* idx, int batch, int ncol, float* dst) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= (long long)batch * ncol) return;
  const long long r = i / ncol, c = i % ncol;
  dst[i] = src[idx[r] * ncol + c];
}

// the loss partials of one batch summed in FP64 into out[0] (one block of 256 threads),
// so that an epoch keeps every batch's loss on the device until its end
__global__ void k_loss_total(const float* part, int n, double* out) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += part[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sh[0];
}

__global__ void k_fill_pattern(bf16* a, long long n, int salt) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) a[i] = __float2bfloat16_rn((float)((i * 2654435761LL + salt) % 2001 - 1000) * 1e-3f);
}

inline unsigned blocks(long long n, int t = 256) { return (unsigned)((n + t - 1) / t); }

}  // namespace emu

using namespace emu;

struct lgame_emu {
  int nlev = 0, nin = 0, nin_pad = 0, hidden = 0, nout = 0, nout_pad = 0, bmax = 0, device = 0;
  cudaStream_t st = nullptr;
  std::vector<void*> allocs;
  int rows[4], cols[4];              // layer l: rows = outputs (padded), cols = inputs (padded)
  float *W[4], *b[4], *gW[4], *gb[4], *mW[4], *vW[4], *mb[4], *vb[4];
  bf16 *Wb[4], *WTb[4];
  float *xmean, *xistd, *ymean, *ystd, *yistd;
  float *xraw, *yraw, *Yt, *Y, *Z[3], *dZ32[4], *part, *lpart, *cpart, *yout;
  bf16 *X, *XT, *H[3], *HT[3], *dZb[4], *dZT[4];
  int* err = nullptr;
  long long adam_t = 0;
  int splits = 32;
  // dataset on the device
  float *dsx = nullptr, *dsy = nullptr;
  long long dsn = 0;
  long long* idx = nullptr;  // one epoch's shuffled order (dsn entries)
  double* lsum = nullptr;    // per-batch loss sums of one epoch (dsn / 128 entries)
  // statistics
  long long gemm_launches = 0;
  double gemm_flop = 0.0;
};

namespace {

int emu_fail(int code, const std::string& msg) {
  lgame_set_error(msg.c_str());
  return code;
}
#define ECK(call)                                                                                    \
  do {                                                                                               \
    cudaError_t e_ = (call);                                                                         \
    if (e_ != cudaSuccess) return emu_fail(LGAME_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <class T>
int ealloc(lgame_emu* e, T** p, size_t n) {
  void* q = nullptr;
  if (cudaMalloc(&q, n * sizeof(T)) != cudaSuccess) return emu_fail(LGAME_ERR_ALLOC, "emulator: cudaMalloc failed");
  if (cudaMemset(q, 0, n * sizeof(T)) != cudaSuccess) return emu_fail(LGAME_ERR_CUDA, "emulator: cudaMemset failed");
  e->allocs.push_back(q);
  *p = (T*)q;
  return LGAME_OK;
}

int check_err(lgame_emu* e) {
  int h = 0;
  ECK(cudaMemcpyAsync(&h, e->err, sizeof(int), cudaMemcpyDeviceToHost, e->st));
  ECK(cudaStreamSynchronize(e->st));
  if (h) return emu_fail(LGAME_ERR_CUDA, "emulator: a tensor-core GEMM timed out waiting for its mbarrier");
  return LGAME_OK;
}

int gemm(lgame_emu* e, const bf16* A, int lda, const bf16* B, int ldb, int M, int N, int K, int splits, const Epi& ep) {
  const int rc = launch_gemm(A, lda, B, ldb, M, N, K, splits, ep, e->err, e->st);
  if (rc != LGAME_OK) return emu_fail(rc, "emulator: GEMM launch failed");
  e->gemm_launches++;
  e->gemm_flop += 2.0 * M * N * (double)K;
  return LGAME_OK;
}

// forward pass of `batch` prepared rows (X, XT); output Y (standardised, padded)
// infer: only the BF16 activations each layer feeds the next (no FP32 pre-activations and
// no transposed copies, which only the backward pass reads)
int forward(lgame_emu* e, int batch, bool infer = false) {
  const int Hd = e->hidden;
  const bf16* in = e->X;
  int ldin = e->nin_pad;
  for (int l = 0; l < 3; ++l) {
    Epi ep{};
    ep.kind = infer ? kEpiBiasGeluH : kEpiBiasGelu;
    ep.bias = e->b[l];
    ep.c = e->Z[l];
    ep.ldc = Hd;
    ep.h = e->H[l];
    ep.ldh = Hd;
    ep.ht = e->HT[l];
    ep.ldt = batch;
    int rc = gemm(e, in, ldin, e->Wb[l], e->cols[l], batch, Hd, e->cols[l], 1, ep);
    if (rc) return rc;
    in = e->H[l];
    ldin = Hd;
  }
  Epi ep{};
  ep.kind = kEpiBias;
  ep.bias = e->b[3];
  ep.c = e->Y;
  ep.ldc = e->nout_pad;
  return gemm(e, in, Hd, e->Wb[3], Hd, batch, e->nout_pad, Hd, 1, ep);
}

// prepared inputs of `batch` rows (a multiple of 128) from raw rows the GPU can read (device
// memory or page-locked host memory), of which the first `valid` hold data
int prep_x(lgame_emu* e, const float* xraw_dev, int batch, int valid, bool infer = false) {
  k_prep_x<<<dim3(e->nin_pad / 32, batch / 32), dim3(32, 8), 0, e->st>>>(xraw_dev, e->nin, e->nin_pad, batch, valid,
                                                                        e->xmean, e->xistd, e->X,
                                                                        infer ? nullptr : e->XT);
  ECK(cudaGetLastError());
  return LGAME_OK;
}

// loss and gradients of one prepared batch (X, XT, Yt); grads in gW, gb; loss partials in lpart
int backward(lgame_emu* e, int batch, int* nparts) {
  const int Hd = e->hidden, no = e->nout_pad;
  const int np = (no / 32) * (batch / 32);
  k_loss_dy<<<dim3(no / 32, batch / 32), dim3(32, 8), 0, e->st>>>(e->Y, e->Yt, e->nout, no, batch, e->dZ32[3], e->dZb[3],
                                                                  e->dZT[3], e->lpart);
  ECK(cudaGetLastError());
  *nparts = np;
  for (int l = 3; l >= 0; --l) {
    // dW_l^T (in x out) = act_{l-1}^T (in x batch) * dZ_l^T (out x batch)^T, split over the batch
    const bf16* actT = (l == 0) ? e->XT : e->HT[l - 1];
    const int nin_l = e->cols[l], nout_l = e->rows[l];
    Epi ep{};
    ep.kind = kEpiF32;
    ep.c = e->part;
    ep.ldc = nout_l;
    ep.split_stride = (long long)nin_l * nout_l;
    const int splits = std::min(e->splits, batch / 64);
    int rc = gemm(e, actT, batch, e->dZT[l], batch, nin_l, nout_l, batch, splits, ep);
    if (rc) return rc;
    const int kchunk = ((batch / splits + 63) / 64) * 64;
    const int zs = (batch + kchunk - 1) / kchunk;
    k_splitk_reduce_t<<<blocks((long long)nin_l * nout_l), 256, 0, e->st>>>(e->part, zs, nin_l, nout_l, e->gW[l]);
    ECK(cudaGetLastError());
    const int chunks = batch / 128;  // rows per chunk: 128
    k_colsum_part<<<dim3(nout_l / 32, chunks), dim3(32, 8), 0, e->st>>>(e->dZ32[l], batch, nout_l, e->cpart);
    k_colsum_fin<<<blocks(nout_l), 256, 0, e->st>>>(e->cpart, chunks, nout_l, e->gb[l]);
    ECK(cudaGetLastError());
    if (l == 0) break;
    // dZ_{l-1} = (dZ_l * W_l) .* gelu'(Z_{l-1}): A = dZ_l (batch x out), B = W_l^T (in x out)
    Epi eb{};
    eb.kind = kEpiGeluBwd;
    eb.zprev = e->Z[l - 1];
    eb.c = e->dZ32[l - 1];
    eb.ldc = Hd;
    eb.h = e->dZb[l - 1];
    eb.ldh = Hd;
    eb.ht = e->dZT[l - 1];
    eb.ldt = batch;
    rc = gemm(e, e->dZb[l], nout_l, e->WTb[l], nout_l, batch, Hd, nout_l, 1, eb);
    if (rc) return rc;
  }
  return LGAME_OK;
}

int adam(lgame_emu* e, float lr) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  e->adam_t++;
  const float c1 = (float)(1.0 / (1.0 - std::pow(0.9, (double)e->adam_t)));
  const float c2 = (float)(1.0 / (1.0 - std::pow(0.999, (double)e->adam_t)));
  for (int l = 0; l < 4; ++l) {
    const long long n = (long long)e->rows[l] * e->cols[l];
    k_adam<<<blocks(n), 256, 0, e->st>>>(e->W[l], e->gW[l], e->mW[l], e->vW[l], n, e->cols[l], lr, b1, b2, c1, c2, eps,
                                         e->Wb[l], e->WTb[l], e->rows[l]);
    k_adam<<<blocks(e->rows[l]), 256, 0, e->st>>>(e->b[l], e->gb[l], e->mb[l], e->vb[l], e->rows[l], 1, lr, b1, b2, c1,
                                                  c2, eps, nullptr, nullptr, 1);
    ECK(cudaGetLastError());
  }
  return LGAME_OK;
}

int loss_from_parts(lgame_emu* e, int nparts, int batch, float* loss) {
  std::vector<float> h(nparts);
  ECK(cudaMemcpyAsync(h.data(), e->lpart, sizeof(float) * nparts, cudaMemcpyDeviceToHost, e->st));
  ECK(cudaStreamSynchronize(e->st));
  double s = 0.0;
  for (float v : h) s += v;
  if (loss) *loss = (float)(s / ((double)batch * e->nout));
  return LGAME_OK;
}

int upload_batch(lgame_emu* e, const float* x, const float* y, int batch) {
  ECK(cudaMemcpyAsync(e->xraw, x, sizeof(float) * (size_t)batch * e->nin, cudaMemcpyHostToDevice, e->st));
  int rc = prep_x(e, e->xraw, batch, batch);
  if (rc) return rc;
  if (y) {
    ECK(cudaMemcpyAsync(e->yraw, y, sizeof(float) * (size_t)batch * e->nout, cudaMemcpyHostToDevice, e->st));
    k_prep_y<<<blocks((long long)batch * e->nout_pad), 256, 0, e->st>>>(e->yraw, e->nout, e->nout_pad, batch, e->ymean,
                                                                         e->yistd, e->Yt);
    ECK(cudaGetLastError());
  }
  return LGAME_OK;
}

int refresh_bf16(lgame_emu* e) {
  for (int l = 0; l < 4; ++l) {
    const long long n = (long long)e->rows[l] * e->cols[l];
    k_to_bf16_t<<<blocks(n), 256, 0, e->st>>>(e->W[l], n, e->cols[l], e->rows[l], e->Wb[l], e->WTb[l]);
    ECK(cudaGetLastError());
  }
  return LGAME_OK;
}

}  // namespace

namespace emu {
// device-side inference for the coupling code: n rows of raw features (device) -> heating
// rates (device, n x nout), in batches of bmax
int infer_device(lgame_emu* e, const float* x_dev, long long n, float* y_dev, cudaStream_t st) {
  if (cudaStreamSynchronize(st) != cudaSuccess) return LGAME_ERR_CUDA;
  for (long long r0 = 0; r0 < n; r0 += e->bmax) {
    const int b = (int)std::min<long long>(e->bmax, n - r0);
    const int bp = ((b + 127) / 128) * 128;
    int rc = prep_x(e, x_dev + r0 * e->nin, bp, b, true);
    if (rc) return rc;
    rc = forward(e, bp, true);
    if (rc) return rc;
    k_denorm<<<blocks((long long)b * e->nout), 256, 0, e->st>>>(e->Y, e->nout, e->nout_pad, b, e->ymean, e->ystd,
                                                                 y_dev + r0 * e->nout);
    ECK(cudaGetLastError());
  }
  ECK(cudaStreamSynchronize(e->st));
  return check_err(e);
}
int nin_of(const lgame_emu* e) { return e->nin; }
int nout_of(const lgame_emu* e) { return e->nout; }
int nlev_of(const lgame_emu* e) { return e->nlev; }
}  // namespace emu

extern "C" int lgame_emu_create(int nlev, int hidden, int batch_max, unsigned long long seed, int device,
                                lgame_emu** out) {
  if (!out || nlev < 3 || nlev > LGAME_RAD_NLEV_MAX || hidden < 256 || hidden % 256 || batch_max < 128 ||
      batch_max % 128)
    return emu_fail(LGAME_ERR_INVALID_ARG, "lgame_emu_create: bad arguments (nlev 3..128, hidden % 256, batch_max % 128)");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0 || device < 0 || device >= ndev)
    return emu_fail(LGAME_ERR_NO_DEVICE, "lgame_emu_create: no CUDA device");
  ECK(cudaSetDevice(device));
  cudaDeviceProp prop;
  ECK(cudaGetDeviceProperties(&prop, device));
  if (prop.major != 10 || prop.minor != 3)
    return emu_fail(LGAME_ERR_NO_DEVICE, "lgame_emu_create: the tensor-core kernels need an sm_103 GPU");
  auto* e = new lgame_emu();
  auto fail = [&](int rc) { lgame_emu_destroy(e); return rc; };
  e->nlev = nlev;
  e->nin = 4 * nlev + 2;
  e->nin_pad = ((e->nin + 63) / 64) * 64;
  e->hidden = hidden;
  e->nout = 2 * nlev;
  e->nout_pad = ((e->nout + 63) / 64) * 64;
  e->bmax = batch_max;
  e->device = device;
  if (cudaStreamCreateWithFlags(&e->st, cudaStreamNonBlocking) != cudaSuccess) return fail(LGAME_ERR_CUDA);
  const int Hd = hidden;
  const int rows[4] = {Hd, Hd, Hd, e->nout_pad}, cols[4] = {e->nin_pad, Hd, Hd, Hd};
  int rc;
  for (int l = 0; l < 4; ++l) {
    e->rows[l] = rows[l];
    e->cols[l] = cols[l];
    const size_t n = (size_t)rows[l] * cols[l];
    if ((rc = ealloc(e, &e->W[l], n)) || (rc = ealloc(e, &e->gW[l], n)) || (rc = ealloc(e, &e->mW[l], n)) ||
        (rc = ealloc(e, &e->vW[l], n)) || (rc = ealloc(e, &e->Wb[l], n)) || (rc = ealloc(e, &e->WTb[l], n)) ||
        (rc = ealloc(e, &e->b[l], rows[l])) || (rc = ealloc(e, &e->gb[l], rows[l])) ||
        (rc = ealloc(e, &e->mb[l], rows[l])) || (rc = ealloc(e, &e->vb[l], rows[l])))
      return fail(rc);
  }
  const size_t B = batch_max;
  if ((rc = ealloc(e, &e->xmean, e->nin)) || (rc = ealloc(e, &e->xistd, e->nin)) || (rc = ealloc(e, &e->ymean, e->nout)) ||
      (rc = ealloc(e, &e->ystd, e->nout)) || (rc = ealloc(e, &e->yistd, e->nout)) ||
      (rc = ealloc(e, &e->xraw, B * e->nin)) || (rc = ealloc(e, &e->yraw, B * e->nout)) ||
      (rc = ealloc(e, &e->Yt, B * e->nout_pad)) || (rc = ealloc(e, &e->Y, B * e->nout_pad)) ||
      (rc = ealloc(e, &e->X, B * e->nin_pad)) || (rc = ealloc(e, &e->XT, B * e->nin_pad)) ||
      (rc = ealloc(e, &e->yout, B * e->nout)) || (rc = ealloc(e, &e->err, 1)))
    return fail(rc);
  for (int l = 0; l < 3; ++l)
    if ((rc = ealloc(e, &e->Z[l], B * Hd)) || (rc = ealloc(e, &e->H[l], B * Hd)) || (rc = ealloc(e, &e->HT[l], B * Hd)))
      return fail(rc);
  for (int l = 0; l < 4; ++l) {
    const size_t w = (l == 3) ? e->nout_pad : Hd;
    if ((rc = ealloc(e, &e->dZ32[l], B * w)) || (rc = ealloc(e, &e->dZb[l], B * w)) || (rc = ealloc(e, &e->dZT[l], B * w)))
      return fail(rc);
  }
  size_t pmax = 0;
  for (int l = 0; l < 4; ++l) pmax = std::max(pmax, (size_t)rows[l] * cols[l]);
  if ((rc = ealloc(e, &e->part, pmax * e->splits)) || (rc = ealloc(e, &e->lpart, B * e->nout_pad / 256 + 1)) ||
      (rc = ealloc(e, &e->cpart, (B / 128) * std::max((size_t)Hd, (size_t)e->nout_pad))))
    return fail(rc);
  // identity normalisation, Xavier-uniform weights (splitmix64), zero biases
  std::vector<float> one(std::max(e->nin, e->nout), 1.f);
  ECK(cudaMemcpy(e->xistd, one.data(), sizeof(float) * e->nin, cudaMemcpyHostToDevice));
  ECK(cudaMemcpy(e->ystd, one.data(), sizeof(float) * e->nout, cudaMemcpyHostToDevice));
  ECK(cudaMemcpy(e->yistd, one.data(), sizeof(float) * e->nout, cudaMemcpyHostToDevice));
  uint64_t s = seed ? seed : 0x9E3779B97F4A7C15ull;
  auto next = [&]() {
    s += 0x9E3779B97F4A7C15ull;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) / 9007199254740992.0;
  };
  const int real_in[4] = {e->nin, Hd, Hd, Hd}, real_out[4] = {Hd, Hd, Hd, e->nout};
  for (int l = 0; l < 4; ++l) {
    std::vector<float> w((size_t)rows[l] * cols[l], 0.f);
    const double a = std::sqrt(6.0 / (real_in[l] + real_out[l]));
    for (int r = 0; r < real_out[l]; ++r)
      for (int c = 0; c < real_in[l]; ++c) w[(size_t)r * cols[l] + c] = (float)((2.0 * next() - 1.0) * a);
    ECK(cudaMemcpy(e->W[l], w.data(), sizeof(float) * w.size(), cudaMemcpyHostToDevice));
  }
  if ((rc = refresh_bf16(e))) return fail(rc);
  ECK(cudaStreamSynchronize(e->st));
  *out = e;
  return LGAME_OK;
}

extern "C" void lgame_emu_destroy(lgame_emu* e) {
  if (!e) return;
  if (e->st) cudaStreamSynchronize(e->st);
  for (void* p : e->allocs) cudaFree(p);
  if (e->dsx) cudaFree(e->dsx);
  if (e->dsy) cudaFree(e->dsy);
  if (e->idx) cudaFree(e->idx);
  if (e->lsum) cudaFree(e->lsum);
  if (e->st) cudaStreamDestroy(e->st);
  delete e;
}

extern "C" long long lgame_emu_num_params(const lgame_emu* e) {
  if (!e) return 0;
  const long long H = e->hidden;
  return H * e->nin + H + 2 * (H * H + H) + (long long)e->nout * H + e->nout;
}

namespace {
// walk the real (unpadded) parameters in the public order: fn(device ptr, row length, rows, row stride)
template <class F>
void for_params(lgame_emu* e, F fn) {
  const int real_in[4] = {e->nin, e->hidden, e->hidden, e->hidden};
  const int real_out[4] = {e->hidden, e->hidden, e->hidden, e->nout};
  for (int l = 0; l < 4; ++l) {
    fn(e->W[l], real_in[l], real_out[l], e->cols[l], l, false);
    fn(e->b[l], real_out[l], 1, real_out[l], l, true);
  }
}
}  // namespace

extern "C" int lgame_emu_get_params(lgame_emu* e, float* out) {
  if (!e || !out) return emu_fail(LGAME_ERR_INVALID_ARG, "lgame_emu_get_params: bad arguments");
  size_t off = 0;
  int rc = LGAME_OK;
  for_params(e, [&](float* d, int len, int nrows, int stride, int, bool) {
    if (rc) return;
    if (cudaMemcpy2D(out + off, len * sizeof(float), d, stride * sizeof(float), len * sizeof(float), nrows,
                     cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = emu_fail(LGAME_ERR_CUDA, "lgame_emu_get_params: copy failed");
    off += (size_t)len * nrows;
  });
  return rc;
}

extern "C" int lgame_emu_set_params(lgame_emu* e, const float* in) {
  if (!e || !in) return emu_fail(LGAME_ERR_INVALID_ARG, "lgame_emu_set_params: bad arguments");
  size_t off = 0;
  int rc = LGAME_OK;
  for_params(e, [&](float* d, int len, int nrows, int stride, int, bool) {
    if (rc) return;
    if (cudaMemcpy2D(d, stride * sizeof(float), in + off, len * sizeof(float), len * sizeof(float), nrows,
                     cudaMemcpyHostToDevice) != cudaSuccess)
      rc = emu_fail(LGAME_ERR_CUDA, "lgame_emu_set_params: copy failed");
    off += (size_t)len * nrows;
  });
  if (rc) return rc;
  rc = refresh_bf16(e);
  if (rc) return rc;
  ECK(cudaStreamSynchronize(e->st));
  return LGAME_OK;
}

extern "C" int lgame_emu_set_normalization(lgame_emu* e, const float* xm, const float* xs, const float* ym,
                                           const float* ys) {
  if (!e || !xm || !xs || !ym || !ys) return emu_fail(LGAME_ERR_INVALID_ARG, "lgame_emu_set_normalization: bad arguments");
  std::vector<float> xi(e->nin), yi(e->nout);
  for (int i = 0; i < e->nin; ++i) xi[i] = xs[i] > 0.f ? 1.f / xs[i] : 0.f;
  for (int i = 0; i < e->nout; ++i) yi[i] = ys[i] > 0.f ? 1.f / ys[i] : 0.f;
  ECK(cudaMemcpy(e->xmean, xm, sizeof(float) * e->nin, cudaMemcpyHostToDevice));
  ECK(cudaMemcpy(e->xistd, xi.data(), sizeof(float) * e->nin, cudaMemcpyHostToDevice));
  ECK(cudaMemcpy(e->ymean, ym, sizeof(float) * e->nout, cudaMemcpyHostToDevice));
  ECK(cudaMemcpy(e->ystd, ys, sizeof(float) * e->nout, cudaMemcpyHostToDevice));
  ECK(cudaMemcpy(e->yistd, yi.data(), sizeof(float) * e->nout, cudaMemcpyHostToDevice));
  return LGAME_OK;
}

extern "C" int lgame_emu_loss_grad(lgame_emu* e, const float* x, const float* y, int batch, float* loss, float* grads) {
  if (!e || !x || !y || batch < 128 || batch % 128 || batch > e->bmax)
    return emu_fail(LGAME_ERR_INVALID_ARG, "lgame_emu_loss_grad: bad arguments (batch a multiple of 128 <= batch_max)");
  int rc = upload_batch(e, x, y, batch);
  if (!rc) rc = forward(e, batch);
  int np = 0;
  if (!rc) rc = backward(e, batch, &np);
  if (!rc) rc = loss_from_parts(e, np, batch, loss);
  if (!rc) rc = check_err(e);
  if (rc) return rc;
  if (grads) {
    size_t off = 0;
    const int real_in[4] = {e->nin, e->hidden, e->hidden, e->hidden};
    const int real_out[4] = {e->hidden, e->hidden, e->hidden, e->nout};
    for (int l = 0; l < 4; ++l) {
      ECK(cudaMemcpy2D(grads + off, real_in[l] * sizeof(float), e->gW[l], e->cols[l] * sizeof(float),
                       real_in[l] * sizeof(float), real_out[l], cudaMemcpyDeviceToHost));
      off += (size_t)real_in[l] * real_out[l];
      ECK(cudaMemcpy(grads + off, e->gb[l], sizeof(float) * real_out[l], cudaMemcpyDeviceToHost));
      off += real_out[l];
    }
  }
  return LGAME_OK;
}

extern "C" int lgame_emu_train_step(lgame_emu* e, const float* x, const float* y, int batch, float lr, float* loss) {
  if (!e || !x || !y || batch < 128 || batch % 128 || batch > e->bmax)
    return emu_fail(LGAME_ERR_INVALID_ARG, "lgame_emu_train_step: bad arguments");
  int rc = upload_batch(e, x, y, batch);
  if (!rc) rc = forward(e, batch);
  int np = 0;
  if (!rc) rc = backward(e, batch, &np);
  if (!rc) rc = adam(e, lr);
  if (!rc) rc = loss_from_parts(e, np, batch, loss);
  if (!rc) rc = check_err(e);
  return rc;
}

extern "C" int lgame_emu_set_dataset(lgame_emu* e, const float* x, const float* y, long long n) {
  if (!e || !x || !y || n < e->bmax) return emu_fail(LGAME_ERR_INVALID_ARG, "lgame_emu_set_dataset: bad arguments");
  if (e->dsx) cudaFree(e->dsx);
  if (e->dsy) cudaFree(e->dsy);
  if (e->idx) cudaFree(e->idx);
  if (e->lsum) cudaFree(e->lsum);
  e->dsx = e->dsy = nullptr;
  e->idx = nullptr;
  e->lsum = nullptr;
  ECK(cudaMalloc(&e->dsx, sizeof(float) * (size_t)n * e->nin));
  ECK(cudaMalloc(&e->dsy, sizeof(float) * (size_t)n * e->nout));
  ECK(cudaMalloc(&e->idx, sizeof(long long) * (size_t)n));
  ECK(cudaMalloc(&e->lsum, sizeof(double) * (size_t)(n / 128 + 1)));
  ECK(cudaMemcpy(e->dsx, x, sizeof(float) * (size_t)n * e->nin, cudaMemcpyHostToDevice));
  ECK(cudaMemcpy(e->dsy, y, sizeof(float) * (size_t)n * e->nout, cudaMemcpyHostToDevice));
  e->dsn = n;
  return LGAME_OK;
}

extern "C" int lgame_emu_train_epoch(lgame_emu* e, int batch, float lr, unsigned long long seed, float* mean_loss) {
  if (!e || !e->dsx || batch < 128 || batch % 128 || batch > e->bmax)
    return emu_fail(LGAME_ERR_INVALID_ARG, "lgame_emu_train_epoch: no dataset or bad batch");
  // shuffled order (Fisher-Yates with splitmix64), whole batches only
  std::vector<long long> perm(e->dsn);
  for (long long i = 0; i < e->dsn; ++i) perm[i] = i;
  uint64_t s = seed ^ 0xD1B54A32D192ED03ull;
  auto next = [&]() {
    s += 0x9E3779B97F4A7C15ull;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  };
  for (long long i = e->dsn - 1; i > 0; --i) std::swap(perm[i], perm[(long long)(next() % (uint64_t)(i + 1))]);
  const long long nb = e->dsn / batch;
  // the whole order goes up once and every batch's loss stays on the device: the batches are
  // enqueued back to back with one synchronisation at the end of the epoch
  ECK(cudaMemcpyAsync(e->idx, perm.data(), sizeof(long long) * (size_t)e->dsn, cudaMemcpyHostToDevice, e->st));
  for (long long k = 0; k < nb; ++k) {
    const long long* idx = e->idx + k * batch;
    k_gather_rows<<<blocks((long long)batch * e->nin), 256, 0, e->st>>>(e->dsx, idx, batch, e->nin, e->xraw);
    k_gather_rows<<<blocks((long long)batch * e->nout), 256, 0, e->st>>>(e->dsy, idx, batch, e->nout, e->yraw);
    ECK(cudaGetLastError());
    int rc = prep_x(e, e->xraw, batch, batch);
    if (rc) return rc;
    k_prep_y<<<blocks((long long)batch * e->nout_pad), 256, 0, e->st>>>(e->yraw, e->nout, e->nout_pad, batch, e->ymean,
                                                                         e->yistd, e->Yt);
    rc = forward(e, batch);
    int np = 0;
    if (!rc) rc = backward(e, batch, &np);
    if (!rc) rc = adam(e, lr);
    if (rc) return rc;
    k_loss_total<<<1, 256, 0, e->st>>>(e->lpart, np, e->lsum + k);
    ECK(cudaGetLastError());
  }
  std::vector<double> ls((size_t)nb);
  if (nb) ECK(cudaMemcpyAsync(ls.data(), e->lsum, sizeof(double) * (size_t)nb, cudaMemcpyDeviceToHost, e->st));
  const int rc = check_err(e);  // synchronises the stream
  if (rc) return rc;
  double acc = 0.0;
  for (long long k = 0; k < nb; ++k) acc += (float)(ls[(size_t)k] / ((double)batch * e->nout));
  if (mean_loss) *mean_loss = nb ? (float)(acc / nb) : 0.f;
  return LGAME_OK;
}

// the device address of a host array the GPU can read and write directly (page-locked and
// mapped), or null
void* mapped_view(const void* host) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
    cudaGetLastError();  // an unregistered pointer may leave an error behind
    return nullptr;
  }
  return (a.type == cudaMemoryTypeHost) ? a.devicePointer : nullptr;
}

// Page-locked x and y are read and written by the kernels themselves over the CPU-GPU link
// (no staging copies); other host arrays go through copies to and from device buffers.
extern "C" int lgame_emu_infer(lgame_emu* e, const float* x, long long n, float* y) {
  if (!e || !x || !y || n < 0) return emu_fail(LGAME_ERR_INVALID_ARG, "lgame_emu_infer: bad arguments");
  const float* xv = (const float*)mapped_view(x);
  float* yv = (float*)mapped_view(y);
  for (long long r0 = 0; r0 < n; r0 += e->bmax) {
    const int b = (int)std::min<long long>(e->bmax, n - r0);
    const int bp = ((b + 127) / 128) * 128;
    const float* src = xv ? xv + r0 * e->nin : e->xraw;
    if (!xv)
      ECK(cudaMemcpyAsync(e->xraw, x + r0 * e->nin, sizeof(float) * (size_t)b * e->nin, cudaMemcpyHostToDevice, e->st));
    int rc = prep_x(e, src, bp, b, true);
    if (!rc) rc = forward(e, bp, true);
    if (rc) return rc;
    k_denorm<<<blocks((long long)b * e->nout), 256, 0, e->st>>>(e->Y, e->nout, e->nout_pad, b, e->ymean, e->ystd,
                                                                 yv ? yv + r0 * e->nout : e->yout);
    ECK(cudaGetLastError());
    if (!yv)
      ECK(cudaMemcpyAsync(y + r0 * e->nout, e->yout, sizeof(float) * (size_t)b * e->nout, cudaMemcpyDeviceToHost, e->st));
  }
  ECK(cudaStreamSynchronize(e->st));
  return check_err(e);
}

extern "C" int lgame_emu_gemm_bf16(lgame_emu* e, const unsigned short* a, const unsigned short* b, float* c, int m,
                                   int n, int k) {
  if (!e || !a || !b || !c || m <= 0 || n <= 0 || k <= 0 || m % 128 || k % 64 || n % 64)
    return emu_fail(LGAME_ERR_INVALID_ARG, "lgame_emu_gemm_bf16: bad arguments (M % 128, K % 64, N % 64)");
  bf16 *da = nullptr, *db = nullptr;
  float* dc = nullptr;
  ECK(cudaMalloc(&da, sizeof(bf16) * (size_t)m * k));
  ECK(cudaMalloc(&db, sizeof(bf16) * (size_t)n * k));
  ECK(cudaMalloc(&dc, sizeof(float) * (size_t)m * n));
  int rc = LGAME_OK;
  if (cudaMemcpy(da, a, sizeof(bf16) * (size_t)m * k, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(db, b, sizeof(bf16) * (size_t)n * k, cudaMemcpyHostToDevice) != cudaSuccess)
    rc = emu_fail(LGAME_ERR_CUDA, "lgame_emu_gemm_bf16: upload failed");
  if (!rc) {
    Epi ep{};
    ep.kind = kEpiF32;
    ep.c = dc;
    ep.ldc = n;
    rc = gemm(e, da, k, db, k, m, n, k, 1, ep);
  }
  if (!rc && cudaStreamSynchronize(e->st) != cudaSuccess) rc = emu_fail(LGAME_ERR_CUDA, "lgame_emu_gemm_bf16: kernel failed");
  if (!rc) rc = check_err(e);
  if (!rc && cudaMemcpy(c, dc, sizeof(float) * (size_t)m * n, cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = emu_fail(LGAME_ERR_CUDA, "lgame_emu_gemm_bf16: download failed");
  cudaFree(da);
  cudaFree(db);
  cudaFree(dc);
  return rc;
}

extern "C" int lgame_emu_stats(lgame_emu* e, long long* launches, double* flop) {
  if (!e) return emu_fail(LGAME_ERR_INVALID_ARG, "lgame_emu_stats: null");
  if (launches) *launches = e->gemm_launches;
  if (flop) *flop = e->gemm_flop;
  e->gemm_launches = 0;
  e->gemm_flop = 0.0;
  return LGAME_OK;
}

extern "C" int lgame_emu_time_gemm(lgame_emu* e, int m, int n, int k, int reps, double* ms) {
  if (!e || !ms || m <= 0 || n <= 0 || k <= 0 || m % 128 || k % 64 || n % 64 || reps < 1)
    return emu_fail(LGAME_ERR_INVALID_ARG, "lgame_emu_time_gemm: bad arguments");
  bf16 *da = nullptr, *db = nullptr;
  float* dc = nullptr;
  cudaEvent_t a0 = nullptr, a1 = nullptr;
  int rc = LGAME_OK;
  if (cudaMalloc(&da, sizeof(bf16) * (size_t)m * k) != cudaSuccess || cudaMalloc(&db, sizeof(bf16) * (size_t)n * k) != cudaSuccess ||
      cudaMalloc(&dc, sizeof(float) * (size_t)m * n) != cudaSuccess || cudaEventCreate(&a0) != cudaSuccess ||
      cudaEventCreate(&a1) != cudaSuccess)
    rc = emu_fail(LGAME_ERR_ALLOC, "lgame_emu_time_gemm: allocation failed");
  if (!rc) {
    k_fill_pattern<<<blocks((long long)m * k), 256, 0, e->st>>>(da, (long long)m * k, 1);
    k_fill_pattern<<<blocks((long long)n * k), 256, 0, e->st>>>(db, (long long)n * k, 7);
    Epi ep{};
    ep.kind = kEpiF32;
    ep.c = dc;
    ep.ldc = n;
    rc = gemm(e, da, k, db, k, m, n, k, 1, ep);
    if (!rc) cudaEventRecord(a0, e->st);
    for (int r = 0; r < reps && !rc; ++r) rc = gemm(e, da, k, db, k, m, n, k, 1, ep);
    if (!rc) {
      cudaEventRecord(a1, e->st);
      if (cudaEventSynchronize(a1) != cudaSuccess) rc = emu_fail(LGAME_ERR_CUDA, "lgame_emu_time_gemm: kernel failed");
    }
    if (!rc) rc = check_err(e);
    if (!rc) {
      float t = 0.f;
      cudaEventElapsedTime(&t, a0, a1);
      *ms = t / reps;
    }
  }
  if (a0) cudaEventDestroy(a0);
  if (a1) cudaEventDestroy(a1);
  cudaFree(da);
  cudaFree(db);
  cudaFree(dc);
  return rc;
}
