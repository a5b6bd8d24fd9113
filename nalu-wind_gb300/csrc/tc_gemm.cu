// Forward layer GEMM of the learned preconditioner on the 5th-generation
// tensor cores: out[r, 0:64] = relu(A[r, 0:128] . W), BF16 inputs, FP32
// accumulation in tensor memory, BF16 output.
//
// Persistent CTAs of 4 warps (two per SM) walk the 128-row tiles. A tile of
// A (128 x 128) and W (64 x 128, given transposed, so both operands are
// K-major) sit in shared memory in the no-swizzle canonical layout: 8-row x
// 16-byte core matrices, K-adjacent cores 128 bytes apart (leading byte
// offset) and 8-row groups 2048 bytes apart (stride byte offset), written
// by 16-byte cp.async copies; the next tile is copied into a second buffer
// while the current one computes. One thread issues eight tcgen05.mma
// (M 128, N 64, K 16) into a 64-column TMEM accumulator and commits them to
// an mbarrier; after the wait each warp reads its 32 TMEM lanes (= rows)
// with tcgen05.ld, applies the ReLU and stores BF16 rows. Every wait is
// bounded: on a timeout the kernel records an error, waits once more
// (bounded) for its MMAs, stops, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "nw_internal.h"

namespace nw {
namespace {

constexpr int kTileM = 128;
constexpr int kN = 64;
constexpr int kK = 128;
constexpr int kABytes = kTileM * kK * 2;  // 32 KiB
constexpr int kBBytes = kN * kK * 2;      // 16 KiB
constexpr int kLbo = 128;                 // K-adjacent core matrices
constexpr int kSbo = (kK / 8) * 128;      // 8-row groups (2048 B)
constexpr int kSmem = 2 * kABytes + kBBytes + 128 + 64;
constexpr uint32_t kTmemCols = 64;
constexpr int kWaitLimit = 1 << 20;

__device__ int g_tc_status;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// tcgen05 shared-memory matrix descriptor: start address, leading and
// stride byte offsets (all >> 4), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = uint64_t((addr >> 4) & 0x3FFFu);
  d |= uint64_t((lbo >> 4) & 0x3FFFu) << 16;
  d |= uint64_t((sbo >> 4) & 0x3FFFu) << 32;
  d |= uint64_t(1) << 46;
  return d;
}

// kind::f16 instruction descriptor: D FP32, A and B BF16, both K-major,
// N = 64, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(kN >> 3) << 17) |
                            (uint32_t(kTileM >> 4) << 24);

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (int it = 0; it < kWaitLimit; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ uint32_t pack_bf16_relu(float a, float b) {
  const __nv_bfloat16 x = __float2bfloat16_rn(fmaxf(a, 0.f));
  const __nv_bfloat16 y = __float2bfloat16_rn(fmaxf(b, 0.f));
  return uint32_t(__bfloat16_as_ushort(x)) | (uint32_t(__bfloat16_as_ushort(y)) << 16);
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes)
               : "memory");
}

// One 128-row tile of A into a shared buffer in the canonical layout; rows
// past m are zero-filled (source size 0, nothing is read).
__device__ __forceinline__ void load_tile(uint32_t dst, const uint16_t* __restrict__ a, int64_t r0,
                                          int64_t m, int tid) {
#pragma unroll
  for (int i = 0; i < kTileM * (kK / 8) / 128; ++i) {
    const int q = tid + 128 * i;
    const int row = q >> 4, kg = q & 15;
    const int64_t gr = r0 + row;
    const bool in = gr < m;
    cp_async16(dst + (row >> 3) * kSbo + kg * kLbo + (row & 7) * 16,
               in ? static_cast<const void*>(a + gr * kK + kg * 8) : static_cast<const void*>(a),
               in ? 16u : 0u);
  }
}

// Persistent CTAs over 128-row tiles: W is staged once per CTA, the next
// tile's A is copied (cp.async) into the other shared buffer while the
// current tile's MMAs and epilogue run.
__global__ void __launch_bounds__(128)
    gemm_fwd_tc_k(const uint16_t* __restrict__ a, const uint16_t* __restrict__ wt,
                  uint16_t* __restrict__ out, int64_t m, int ldo) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) &
                                             ~uintptr_t(127));
  uint8_t* sB = base;
  uint8_t* sA0 = base + kBBytes;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sA0 + 2 * kABytes);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mbar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t ntiles = (m + kTileM - 1) / kTileM;
  const uint32_t b0 = smem_u32(sB), a0 = smem_u32(sA0);

  // W (64 x 128) and the first A tile form the first copy group
#pragma unroll
  for (int i = 0; i < kN * (kK / 8) / 128; ++i) {
    const int q = tid + 128 * i;
    const int row = q >> 4, kg = q & 15;
    cp_async16(b0 + (row >> 3) * kSbo + kg * kLbo + (row & 7) * 16, wt + q * 8, 16u);
  }
  if (blockIdx.x < ntiles) load_tile(a0, a, int64_t(blockIdx.x) * kTileM, m, tid);
  asm volatile("cp.async.commit_group;" ::: "memory");

  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const uint32_t bar = smem_u32(mbar);

  int it = 0;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x, ++it) {
    const uint32_t abuf = a0 + uint32_t(it & 1) * kABytes;
    const int64_t tn = t + gridDim.x;
    if (tn < ntiles) load_tile(a0 + uint32_t((it + 1) & 1) * kABytes, a, tn * kTileM, m, tid);
    asm volatile("cp.async.commit_group;" ::: "memory");
    asm volatile("cp.async.wait_group 1;" ::: "memory");  // this tile (and W) landed
    // the copies become visible to the tensor cores (async proxy)
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
#pragma unroll
      for (int k = 0; k < kK / 16; ++k) {
        // K step of 16 = two core matrices along K
        const uint64_t da = smem_desc(abuf + k * 2 * kLbo, kLbo, kSbo);
        const uint64_t db = smem_desc(b0 + k * 2 * kLbo, kLbo, kSbo);
        const uint32_t acc = k > 0 ? 1u : 0u;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
            "l"(da), "l"(db), "r"(kIdesc), "r"(acc)
            : "memory");
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              bar)
          : "memory");
    }
    const uint32_t parity = uint32_t(it & 1);
    bool ok = mbar_wait(bar, parity);
    if (!ok) {
      atomicExch(&g_tc_status, 1);
      ok = mbar_wait(bar, parity);  // let the MMAs drain before the TMEM is freed
    }
    if (!__syncthreads_and(ok)) break;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    uint32_t v[64];
    const uint32_t taddr = tmem + (uint32_t(warp * 32) << 16);
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
          "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
          "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]),
          "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
          "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]),
          "=r"(v[31])
        : "r"(taddr));
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(v[32]), "=r"(v[33]), "=r"(v[34]), "=r"(v[35]), "=r"(v[36]), "=r"(v[37]),
          "=r"(v[38]), "=r"(v[39]), "=r"(v[40]), "=r"(v[41]), "=r"(v[42]), "=r"(v[43]),
          "=r"(v[44]), "=r"(v[45]), "=r"(v[46]), "=r"(v[47]), "=r"(v[48]), "=r"(v[49]),
          "=r"(v[50]), "=r"(v[51]), "=r"(v[52]), "=r"(v[53]), "=r"(v[54]), "=r"(v[55]),
          "=r"(v[56]), "=r"(v[57]), "=r"(v[58]), "=r"(v[59]), "=r"(v[60]), "=r"(v[61]),
          "=r"(v[62]), "=r"(v[63])
        : "r"(taddr + 32u));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    const int64_t r = t * kTileM + warp * 32 + lane;
    if (r < m) {
      uint4* dst = reinterpret_cast<uint4*>(out + r * ldo);
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        uint4 o;
        o.x = pack_bf16_relu(__uint_as_float(v[8 * c + 0]), __uint_as_float(v[8 * c + 1]));
        o.y = pack_bf16_relu(__uint_as_float(v[8 * c + 2]), __uint_as_float(v[8 * c + 3]));
        o.z = pack_bf16_relu(__uint_as_float(v[8 * c + 4]), __uint_as_float(v[8 * c + 5]));
        o.w = pack_bf16_relu(__uint_as_float(v[8 * c + 6]), __uint_as_float(v[8 * c + 7]));
        dst[c] = o;
      }
    }
    // every warp has read the accumulator before the next tile's MMAs
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols)
                 : "memory");
  }
}

// ---------------------------------------------------------------------------
// The same layer with the tiles brought in by the Tensor Memory Accelerator:
// cp.async.bulk.tensor copies 128-row x 64-element (128-byte) panels of A
// and W into shared memory with the 128-byte swizzle, which is the layout
// the UMMA descriptors read as SWIZZLE_128B K-major (8-row groups 1024 bytes
// apart; a K step of 16 advances the start address by 32 bytes inside the
// swizzle atom). One thread issues the copies against an mbarrier's
// transaction count; the next tile streams into the other buffer while the
// current one computes. Rows past m are zero-filled by the copy engine.
constexpr int kPanelA = kTileM * 128;  // 16 KiB: 128 rows x 128 bytes
constexpr int kPanelB = kN * 128;      // 8 KiB
constexpr int kSmemTma = 2 * kPanelB + 2 * 2 * kPanelA + 1024 + 64;

__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
  uint64_t d = uint64_t((addr >> 4) & 0x3FFFu);
  d |= uint64_t(1) << 16;                     // leading byte offset (unused for swizzled K-major)
  d |= uint64_t((1024 >> 4) & 0x3FFFu) << 32;  // 8-row groups 1024 bytes apart
  d |= uint64_t(1) << 46;                     // descriptor version
  d |= uint64_t(2) << 61;                     // SWIZZLE_128B
  return d;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
      "[%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

__global__ void __launch_bounds__(128)
    gemm_fwd_tma_k(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_w,
                   uint16_t* __restrict__ out, int64_t m, int ldo) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  uint8_t* sB = base;                    // 2 panels of W
  uint8_t* sA = base + 2 * kPanelB;      // 2 buffers x 2 panels of A
  uint64_t* bars = reinterpret_cast<uint64_t*>(sA + 4 * kPanelA);  // full[2], w, mma
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 4);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t ntiles = (m + kTileM - 1) / kTileM;
  const uint32_t b0 = smem_u32(sB), a0 = smem_u32(sA);
  const uint32_t full0 = smem_u32(bars), wbar = smem_u32(bars + 2), mbar = smem_u32(bars + 3);

  if (tid == 0) {
    for (int i = 0; i < 4; ++i)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bars + i)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    expect_tx(wbar, 2 * kPanelB);
    tma_load_2d(b0, &map_w, 0, 0, wbar);
    tma_load_2d(b0 + kPanelB, &map_w, 64, 0, wbar);
    if (blockIdx.x < ntiles) {
      const int y = int(int64_t(blockIdx.x) * kTileM);
      expect_tx(full0, 2 * kPanelA);
      tma_load_2d(a0, &map_a, 0, y, full0);
      tma_load_2d(a0 + kPanelA, &map_a, 64, y, full0);
    }
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  bool ok = mbar_wait(wbar, 0);
  int it = 0;
  for (int64_t t = blockIdx.x; ok && t < ntiles; t += gridDim.x, ++it) {
    const int bsel = it & 1;
    const uint32_t abuf = a0 + uint32_t(bsel) * 2 * kPanelA;
    const int64_t tn = t + gridDim.x;
    if (tid == 0 && tn < ntiles) {
      // the other buffer was read by the previous tile's MMAs, which completed
      const uint32_t nb = a0 + uint32_t(1 - bsel) * 2 * kPanelA;
      const uint32_t fb = full0 + uint32_t(1 - bsel) * 8;
      const int y = int(tn * kTileM);
      expect_tx(fb, 2 * kPanelA);
      tma_load_2d(nb, &map_a, 0, y, fb);
      tma_load_2d(nb + kPanelA, &map_a, 64, y, fb);
    }
    ok = mbar_wait(full0 + uint32_t(bsel) * 8, uint32_t((it >> 1) & 1));
    if (!__syncthreads_and(ok)) break;
    if (tid == 0) {
#pragma unroll
      for (int k = 0; k < kK / 16; ++k) {
        // panel k / 4, 32-byte step k % 4 inside the 128-byte swizzle atom
        const uint32_t off = uint32_t(k >> 2) * kPanelA + uint32_t(k & 3) * 32;
        const uint32_t offb = uint32_t(k >> 2) * kPanelB + uint32_t(k & 3) * 32;
        const uint64_t da = smem_desc_sw128(abuf + off);
        const uint64_t db = smem_desc_sw128(b0 + offb);
        const uint32_t acc = k > 0 ? 1u : 0u;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
            "l"(da), "l"(db), "r"(kIdesc), "r"(acc)
            : "memory");
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
          : "memory");
    }
    ok = mbar_wait(mbar, uint32_t(it & 1));
    if (!ok) {
      atomicExch(&g_tc_status, 1);
      ok = mbar_wait(mbar, uint32_t(it & 1));
    }
    if (!__syncthreads_and(ok)) break;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    uint32_t v[64];
    const uint32_t taddr = tmem + (uint32_t(warp * 32) << 16);
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
          "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
          "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]),
          "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
          "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]),
          "=r"(v[31])
        : "r"(taddr));
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(v[32]), "=r"(v[33]), "=r"(v[34]), "=r"(v[35]), "=r"(v[36]), "=r"(v[37]),
          "=r"(v[38]), "=r"(v[39]), "=r"(v[40]), "=r"(v[41]), "=r"(v[42]), "=r"(v[43]),
          "=r"(v[44]), "=r"(v[45]), "=r"(v[46]), "=r"(v[47]), "=r"(v[48]), "=r"(v[49]),
          "=r"(v[50]), "=r"(v[51]), "=r"(v[52]), "=r"(v[53]), "=r"(v[54]), "=r"(v[55]),
          "=r"(v[56]), "=r"(v[57]), "=r"(v[58]), "=r"(v[59]), "=r"(v[60]), "=r"(v[61]),
          "=r"(v[62]), "=r"(v[63])
        : "r"(taddr + 32u));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    const int64_t r = t * kTileM + warp * 32 + lane;
    if (r < m) {
      uint4* dst = reinterpret_cast<uint4*>(out + r * ldo);
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        uint4 o;
        o.x = pack_bf16_relu(__uint_as_float(v[8 * c + 0]), __uint_as_float(v[8 * c + 1]));
        o.y = pack_bf16_relu(__uint_as_float(v[8 * c + 2]), __uint_as_float(v[8 * c + 3]));
        o.z = pack_bf16_relu(__uint_as_float(v[8 * c + 4]), __uint_as_float(v[8 * c + 5]));
        o.w = pack_bf16_relu(__uint_as_float(v[8 * c + 6]), __uint_as_float(v[8 * c + 7]));
        dst[c] = o;
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  }
  if (!ok) atomicExch(&g_tc_status, 1);
  // copies still in flight (a prefetched tile after an early stop) land
  // before the shared memory is released: wait for both buffers (bounded)
  if (tid == 0 && !ok) {
    mbar_wait(full0, uint32_t(((it + 1) >> 1) & 1));
    mbar_wait(full0 + 8, uint32_t((it >> 1) & 1));
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols)
                 : "memory");
  }
}

// ---------------------------------------------------------------------------
// Backward layer GEMMs of the training step on the tcgen05 tensor cores.
//
// dX = dZ W^T: dx[r, 0:128] (FP32) = dz[r, 0:64] . w[0:128, 0:64]^T. Both
// operands are K-major (K = 64 output channels, 128 bytes per row: one
// swizzle-128B atom wide), loaded by TMA; M 128, N 128, four K16 steps into
// a 128-column TMEM accumulator; persistent CTAs over 128-row tiles with
// the next dz tile streaming into the other buffer.
constexpr int kDxN = 128;
constexpr int kDxPanel = kTileM * 128;      // 16 KiB: 128 rows x 64 BF16
constexpr int kSmemDx = 3 * kDxPanel + 1024 + 64;
constexpr uint32_t kIdescDx = (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(kDxN >> 3) << 17) |
                              (uint32_t(kTileM >> 4) << 24);

// 32 columns of this warp's 32 TMEM lanes as FP32
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* f) {
  uint32_t v[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
        "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]),
        "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
        "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]),
        "=r"(v[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) f[i] = __uint_as_float(v[i]);
}

__global__ void __launch_bounds__(128)
    gemm_dx_tma_k(const __grid_constant__ CUtensorMap map_dz, const __grid_constant__ CUtensorMap map_w,
                  float* __restrict__ dx, int64_t m) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  uint8_t* sW = base;                   // w (128 x 64)
  uint8_t* sA = base + kDxPanel;        // 2 buffers of dz tiles
  uint64_t* bars = reinterpret_cast<uint64_t*>(sA + 2 * kDxPanel);  // full[2], w, mma
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 4);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t ntiles = (m + kTileM - 1) / kTileM;
  const uint32_t w0 = smem_u32(sW), a0 = smem_u32(sA);
  const uint32_t full0 = smem_u32(bars), wbar = smem_u32(bars + 2), mbar = smem_u32(bars + 3);
  if (tid == 0) {
    for (int i = 0; i < 4; ++i)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bars + i)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    expect_tx(wbar, kDxPanel);
    tma_load_2d(w0, &map_w, 0, 0, wbar);
    if (blockIdx.x < ntiles) {
      expect_tx(full0, kDxPanel);
      tma_load_2d(a0, &map_dz, 0, int(int64_t(blockIdx.x) * kTileM), full0);
    }
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(uint32_t(kDxN))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  bool ok = mbar_wait(wbar, 0);
  int it = 0;
  for (int64_t t = blockIdx.x; ok && t < ntiles; t += gridDim.x, ++it) {
    const int bsel = it & 1;
    const uint32_t abuf = a0 + uint32_t(bsel) * kDxPanel;
    const int64_t tn = t + gridDim.x;
    if (tid == 0 && tn < ntiles) {
      // the other buffer was read by the previous tile's MMAs, which completed
      const uint32_t fb = full0 + uint32_t(1 - bsel) * 8;
      expect_tx(fb, kDxPanel);
      tma_load_2d(a0 + uint32_t(1 - bsel) * kDxPanel, &map_dz, 0, int(tn * kTileM), fb);
    }
    ok = mbar_wait(full0 + uint32_t(bsel) * 8, uint32_t((it >> 1) & 1));
    if (!__syncthreads_and(ok)) break;
    if (tid == 0) {
#pragma unroll
      for (int k = 0; k < 4; ++k) {  // 32-byte K16 steps inside the swizzle atom
        const uint64_t da = smem_desc_sw128(abuf + uint32_t(k) * 32);
        const uint64_t db = smem_desc_sw128(w0 + uint32_t(k) * 32);
        const uint32_t acc = k > 0 ? 1u : 0u;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
            "l"(da), "l"(db), "r"(kIdescDx), "r"(acc)
            : "memory");
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
          : "memory");
    }
    ok = mbar_wait(mbar, uint32_t(it & 1));
    if (!ok) {
      atomicExch(&g_tc_status, 1);
      ok = mbar_wait(mbar, uint32_t(it & 1));
    }
    if (!__syncthreads_and(ok)) break;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int64_t r = t * kTileM + warp * 32 + lane;
    const uint32_t taddr = tmem + (uint32_t(warp * 32) << 16);
#pragma unroll
    for (int h = 0; h < kDxN / 32; ++h) {
      float f[32];
      tmem_ld32(taddr + uint32_t(32 * h), f);
      if (r < m) {
        float4* dst = reinterpret_cast<float4*>(dx + r * kDxN + 32 * h);
#pragma unroll
        for (int c = 0; c < 8; ++c) dst[c] = make_float4(f[4 * c], f[4 * c + 1], f[4 * c + 2], f[4 * c + 3]);
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  }
  if (!ok) atomicExch(&g_tc_status, 1);
  if (tid == 0 && !ok) {
    mbar_wait(full0, uint32_t(((it + 1) >> 1) & 1));
    mbar_wait(full0 + 8, uint32_t((it >> 1) & 1));
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(uint32_t(kDxN))
                 : "memory");
  }
}

// dW partials: partial[block][c][o] = sum over this block's nodes of
// x[node][c] dz[node][o] (c < 128, o < 64). The reduction runs over nodes,
// which both operands store as rows, so each 64-node chunk is transposed
// while it is staged: x^T (128 x 64) and dz^T (64 x 64) in the no-swizzle
// K-major canonical layout (8-row x 16-byte core matrices, K-adjacent cores
// 128 bytes apart, 8-row groups 1024 bytes apart), built from pairs of
// node rows so that each shared store is one 32-bit word. Four K16 MMAs (M
// 128, N 64) per chunk accumulate in TMEM over the block's chunks (grid
// stride); one commit-and-wait per chunk frees the staging buffer.
constexpr int kWgChunk = 64;
constexpr int kWgSbo = (kWgChunk / 8) * 128;  // 1024
constexpr int kWgABytes = 128 * kWgChunk * 2;  // 16 KiB
constexpr int kWgBBytes = 64 * kWgChunk * 2;   // 8 KiB
constexpr int kSmemWg = kWgABytes + kWgBBytes + 128 + 64;

// word offset of the element pair (row, k), (row, k + 1) in a canonical tile
__device__ __forceinline__ uint32_t wg_off(int row, int k) {
  return uint32_t((row >> 3) * kWgSbo + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

__global__ void __launch_bounds__(128)
    gemm_wgrad_tc_k(const uint16_t* __restrict__ xc, const uint16_t* __restrict__ dz,
                    float* __restrict__ partial, int64_t m) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) &
                                             ~uintptr_t(127));
  uint8_t* sA = base;
  uint8_t* sB = base + kWgABytes;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sB + kWgBBytes);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mbar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB), bar = smem_u32(mbar);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  bool ok = true, any = false;
  int it = 0;
  // thread -> k pair (lane: nodes 2 kp, 2 kp + 1) and column groups of 8
  const int kp = lane;
  for (int64_t c0 = int64_t(blockIdx.x) * kWgChunk; ok && c0 < m;
       c0 += int64_t(gridDim.x) * kWgChunk, ++it) {
    const int64_t n0 = c0 + 2 * kp, n1 = n0 + 1;
    // x: 16 groups of 8 columns, 4 per warp
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int cg = warp + 4 * i;
      uint4 u0 = make_uint4(0, 0, 0, 0), u1 = u0;
      if (n0 < m) u0 = *reinterpret_cast<const uint4*>(xc + n0 * 128 + cg * 8);
      if (n1 < m) u1 = *reinterpret_cast<const uint4*>(xc + n1 * 128 + cg * 8);
      const uint32_t w0[4] = {u0.x, u0.y, u0.z, u0.w}, w1[4] = {u1.x, u1.y, u1.z, u1.w};
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        // columns 8 cg + 2 j (low halves) and 8 cg + 2 j + 1 (high halves)
        const uint32_t lo = (w0[j] & 0xffffu) | (w1[j] << 16);
        const uint32_t hi = (w0[j] >> 16) | (w1[j] & 0xffff0000u);
        const int c = 8 * cg + 2 * j;
        asm volatile("st.shared.b32 [%0], %1;" ::"r"(a0 + wg_off(c, 2 * kp)), "r"(lo) : "memory");
        asm volatile("st.shared.b32 [%0], %1;" ::"r"(a0 + wg_off(c + 1, 2 * kp)), "r"(hi) : "memory");
      }
    }
    // dz: 8 groups of 8 columns, 2 per warp
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const int cg = warp + 4 * i;
      uint4 u0 = make_uint4(0, 0, 0, 0), u1 = u0;
      if (n0 < m) u0 = *reinterpret_cast<const uint4*>(dz + n0 * 64 + cg * 8);
      if (n1 < m) u1 = *reinterpret_cast<const uint4*>(dz + n1 * 64 + cg * 8);
      const uint32_t w0[4] = {u0.x, u0.y, u0.z, u0.w}, w1[4] = {u1.x, u1.y, u1.z, u1.w};
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const uint32_t lo = (w0[j] & 0xffffu) | (w1[j] << 16);
        const uint32_t hi = (w0[j] >> 16) | (w1[j] & 0xffff0000u);
        const int c = 8 * cg + 2 * j;
        asm volatile("st.shared.b32 [%0], %1;" ::"r"(b0 + wg_off(c, 2 * kp)), "r"(lo) : "memory");
        asm volatile("st.shared.b32 [%0], %1;" ::"r"(b0 + wg_off(c + 1, 2 * kp)), "r"(hi) : "memory");
      }
    }
    // the stores become visible to the tensor cores (async proxy)
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
#pragma unroll
      for (int k = 0; k < kWgChunk / 16; ++k) {
        const uint64_t da = smem_desc(a0 + uint32_t(k) * 256, 128, kWgSbo);
        const uint64_t db = smem_desc(b0 + uint32_t(k) * 256, 128, kWgSbo);
        const uint32_t acc = (it > 0 || k > 0) ? 1u : 0u;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
            "l"(da), "l"(db), "r"(kIdesc), "r"(acc)
            : "memory");
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
          : "memory");
    }
    // the staging buffer is reused by the next chunk once the MMAs read it
    ok = mbar_wait(bar, uint32_t(it & 1));
    if (!ok) {
      atomicExch(&g_tc_status, 1);
      ok = mbar_wait(bar, uint32_t(it & 1));
    }
    ok = __syncthreads_and(ok) != 0;
    any = true;
  }
  if (!ok) atomicExch(&g_tc_status, 1);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  // rows of D are input channels c (TMEM lanes), columns output channels
  float* out = partial + int64_t(blockIdx.x) * (128 * 64) + int64_t(warp * 32 + lane) * 64;
  const uint32_t taddr = tmem + (uint32_t(warp * 32) << 16);
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    float f[32];
    tmem_ld32(taddr + uint32_t(32 * h), f);
    float4* dst = reinterpret_cast<float4*>(out + 32 * h);
#pragma unroll
    for (int c = 0; c < 8; ++c)
      dst[c] = (any && ok) ? make_float4(f[4 * c], f[4 * c + 1], f[4 * c + 2], f[4 * c + 3])
                           : make_float4(0.f, 0.f, 0.f, 0.f);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols)
                 : "memory");
  }
}

}  // namespace

void launch_gemm_fwd_tc(const uint16_t* a, const uint16_t* wt, uint16_t* out, int64_t m,
                        int ldo, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    NW_CUDA(cudaFuncSetAttribute(gemm_fwd_tc_k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 kSmem));
    attr = true;
  }
  static int ctas = 0;
  if (!ctas) {
    int dev = 0, sms = 0;
    NW_CUDA(cudaGetDevice(&dev));
    NW_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    ctas = 2 * sms;  // two 80 KiB CTAs per SM
  }
  if (m <= 0) return;
  const int64_t tiles = (m + kTileM - 1) / kTileM;
  const unsigned grid = unsigned(tiles < ctas ? tiles : ctas);
  gemm_fwd_tc_k<<<grid, 128, kSmem, s>>>(a, wt, out, m, ldo);
  NW_CUDA(cudaGetLastError());
}

// Tensor maps of the TMA variant (cuTensorMapEncodeTiled through the
// runtime's driver entry point: no link against the driver library).
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                   const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    NW_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !p) fail(NW_CUDA_ERROR, "cuTensorMapEncodeTiled unavailable");
    fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}
// rows x cols BF16 (row stride 2 cols bytes), boxes of 128 bytes x box_rows
static CUtensorMap make_map(const uint16_t* base, int64_t rows, uint32_t box_rows, int cols = kK) {
  CUtensorMap map;
  const cuuint64_t dims[2] = {cuuint64_t(cols), cuuint64_t(rows)};
  const cuuint64_t strides[1] = {cuuint64_t(cols) * 2};
  const cuuint32_t box[2] = {64, box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = encode_fn()(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                                 const_cast<uint16_t*>(base), dims, strides, box, estr,
                                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                 CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) fail(NW_INVALID_ARG, "tensor map encoding failed");
  return map;
}

void launch_gemm_fwd_tma(const uint16_t* a, const uint16_t* wt, uint16_t* out, int64_t m, int ldo,
                         cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    NW_CUDA(cudaFuncSetAttribute(gemm_fwd_tma_k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 kSmemTma));
    attr = true;
  }
  static int ctas = 0;
  if (!ctas) {
    int dev = 0, sms = 0;
    NW_CUDA(cudaGetDevice(&dev));
    NW_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    ctas = 2 * sms;
  }
  if (m <= 0) return;
  if ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(wt)) & 15u)
    fail(NW_INVALID_ARG, "TMA operands must be 16-byte aligned");
  const CUtensorMap ma = make_map(a, m, kTileM);
  const CUtensorMap mw = make_map(wt, kN, kN);
  const int64_t tiles = (m + kTileM - 1) / kTileM;
  const unsigned grid = unsigned(tiles < ctas ? tiles : ctas);
  gemm_fwd_tma_k<<<grid, 128, kSmemTma, s>>>(ma, mw, out, m, ldo);
  NW_CUDA(cudaGetLastError());
}

void launch_gemm_dx_tma(const uint16_t* dz, const uint16_t* w, float* dx, int64_t m,
                        cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    NW_CUDA(cudaFuncSetAttribute(gemm_dx_tma_k, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemDx));
    attr = true;
  }
  static int ctas = 0;
  if (!ctas) {
    int dev = 0, sms = 0;
    NW_CUDA(cudaGetDevice(&dev));
    NW_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    ctas = 2 * sms;
  }
  if (m <= 0) return;
  if ((reinterpret_cast<uintptr_t>(dz) | reinterpret_cast<uintptr_t>(w) |
       reinterpret_cast<uintptr_t>(dx)) & 15u)
    fail(NW_INVALID_ARG, "TMA operands must be 16-byte aligned");
  const CUtensorMap mz = make_map(dz, m, kTileM, 64);
  const CUtensorMap mw = make_map(w, kDxN, kDxN, 64);
  const int64_t tiles = (m + kTileM - 1) / kTileM;
  const unsigned grid = unsigned(tiles < ctas ? tiles : ctas);
  gemm_dx_tma_k<<<grid, 128, kSmemDx, s>>>(mz, mw, dx, m);
  NW_CUDA(cudaGetLastError());
}

void launch_wgrad_partials_tc(const uint16_t* xc, const uint16_t* dz, float* partial, int64_t m,
                              int blocks, cudaStream_t s) {
  if (blocks <= 0) return;
  if ((reinterpret_cast<uintptr_t>(xc) | reinterpret_cast<uintptr_t>(dz) |
       reinterpret_cast<uintptr_t>(partial)) & 15u)
    fail(NW_INVALID_ARG, "GEMM operands must be 16-byte aligned");
  gemm_wgrad_tc_k<<<blocks, 128, kSmemWg, s>>>(xc, dz, partial, m);
  NW_CUDA(cudaGetLastError());
}

// Reads and clears the timeout flag of the tensor-core kernels (stream
// ordered; synchronises the stream).
int tc_status(cudaStream_t s) {
  int v = 0;
  NW_CUDA(cudaMemcpyFromSymbolAsync(&v, g_tc_status, sizeof(int), 0, cudaMemcpyDeviceToHost, s));
  const int zero = 0;
  NW_CUDA(cudaMemcpyToSymbolAsync(g_tc_status, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, s));
  NW_CUDA(cudaStreamSynchronize(s));
  return v;
}

}  // namespace nw
