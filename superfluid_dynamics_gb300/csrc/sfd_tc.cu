// sfd_tc.cu -- tensor-core (tcgen05) trailing update of the blocked
// Gauss-Jordan preconditioner.
//
// Step kb of the in-place Gauss-Jordan inverse updates every 128 x 128 tile
// (i, j) outside block row / column K:
//     A_ij -= C_i R_j,   C_i = A_iK (128 x 128),  R_j = P A_Kj (128 x 128)
// a K = 128 GEMM per tile.  The panel kernel stores C and R^T split into three
// bf16 parts (x = hi + mid + lo: hi = bf16(x), mid = bf16(x - hi),
// lo = bf16(x - hi - mid); 24 significant bits, an FP32 value), K-major.  Each
// CTA:
//   1. copies its six operand tiles (C and R^T, three parts each, 32 KB each)
//      into shared memory with cp.async in the 128-byte-swizzled K-major
//      layout the tensor core reads (8-row x 128-byte atoms, chunk ^= row % 8);
//   2. one thread issues 6 x 8 tcgen05.mma (kind::f16, M = N = 128, K = 16)
//      accumulating the six products of order >= 2^-24 (hi.hi, hi.mid, mid.hi,
//      hi.lo, mid.mid, lo.hi) in FP32 in tensor memory, and commits them to an
//      mbarrier;
//   3. four warps read the accumulator back with tcgen05.ld (one row per
//      thread) and subtract it from A_ij in global memory.
// The result carries FP32-level error (~2^-24 relative per product), so the
// FP32 refinement corrections that follow stay small.
//
// Every wait is bounded: a spin that runs out sets SFD_ST_TIMEOUT in the
// surface status, skips the epilogue, still frees its tensor memory and
// returns.
#include <cuda_bf16.h>

#include "sfd_engine.cuh"
#include "sfd_solve.cuh"

namespace {

constexpr int kTile = 128;                     // M = N = K of one tile update
constexpr int kOpBytes = kTile * kTile * 2;    // one bf16 operand tile (32 KB)
constexpr int kParts = 3;                      // bf16 parts per operand
constexpr int kTcThreads = 128;
constexpr unsigned kSpinLimit = 1u << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor (tcgen05 format): start address, leading
// byte offset (unused for swizzled K-major: 16 B), stride byte offset (1024 B
// between 8-row atoms), version 1, layout SWIZZLE_128B (2).
__device__ __forceinline__ uint64_t make_sdesc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)(16 >> 4) << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// Instruction descriptor: kind::f16, D = F32, A = B = BF16, both K-major,
// N = 128 (N >> 3 at bit 17), M = 128 (M >> 4 at bit 24).
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTile >> 3) << 17) |
                            ((uint32_t)(kTile >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(kIdesc), "r"(acc));
}

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
  for (unsigned it = 0; it < kSpinLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Copy a 128 x 128 bf16 K-major tile (rows of 256 B, row stride `ld` elements)
// into the swizzled layout: two K-halves of 16 KB, each 128 rows x 128 B.
__device__ __forceinline__ void load_tile_async(uint32_t sbase, const __nv_bfloat16* g, int ld) {
  for (int e = threadIdx.x; e < kTile * 16; e += kTcThreads) {
    int r = e >> 4, c16 = e & 15;          // row, 16-byte chunk along K
    int half = c16 >> 3, c = c16 & 7;
    uint32_t dst = sbase + half * (kTile * 128) + r * 128 + ((c ^ (r & 7)) << 4);
    const void* src = g + (long long)r * ld + c16 * 8;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src) : "memory");
  }
}

}  // namespace

// Grid (tiles, tiles, nsurf) over 128 x 128 tiles; tiles in block row or column
// K return at once (the SIMT kernel handles those).
__global__ void __launch_bounds__(kTcThreads, 1)
    k_gj_update_tc(const SurfaceDesc* surf, int kb, float* mat, const __nv_bfloat16* cparts,
                   const __nv_bfloat16* rparts, long long part_stride, const long long* poff, unsigned int* status) {
  const int s = blockIdx.z;
  const SurfaceDesc& S = surf[s];
  const int np = pad_n(S.n), kt = kb;  // block K = tile row/column kb (128 wide)
  const int ti = blockIdx.y, tj = blockIdx.x;
  if (kt * kTile >= np || ti * kTile >= np || tj * kTile >= np) return;
  if (ti == kt || tj == kt) return;
  extern __shared__ uint8_t tc_smem_raw[];
  // operand tiles need 1024-byte alignment for the 128-byte swizzle
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~uintptr_t(1023));
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base_sh;
  const uint32_t sA = smem_u32(base), sB = sA + kParts * kOpBytes;  // parts p at + p * kOpBytes
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  // tensor memory: 128 columns of FP32 accumulator (128 lanes = rows)
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_base_sh)),
                 "r"(kTile));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;\n");
  }
  // operands: C rows ti*128.., R^T rows tj*128.. (both K-major, ld = 128)
  const long long po = poff[s];
  for (int p = 0; p < kParts; ++p) {
    load_tile_async(sA + p * kOpBytes, cparts + p * part_stride + po + (long long)ti * kTile * kTile, kTile);
    load_tile_async(sB + p * kOpBytes, rparts + p * part_stride + po + (long long)tj * kTile * kTile, kTile);
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_base_sh;

  if (threadIdx.x == 0) {
    uint32_t acc = 0;
    // products with part-index sum <= 2: (hi,hi) (hi,mid) (mid,hi) (hi,lo) (mid,mid) (lo,hi)
    const int pa[6] = {0, 0, 1, 0, 1, 2}, pb[6] = {0, 1, 0, 2, 1, 0};
    for (int p = 0; p < 6; ++p) {
      const uint32_t Ap = sA + pa[p] * kOpBytes, Bp = sB + pb[p] * kOpBytes;
      for (int kk = 0; kk < kTile / 16; ++kk) {
        // K step kk: K-half kk/4 (16 KB apart), 32 bytes per step inside the atom
        uint32_t koff = (uint32_t)(kk >> 2) * (kTile * 128) + (uint32_t)(kk & 3) * 32;
        mma_bf16(tmem, make_sdesc(Ap + koff), make_sdesc(Bp + koff), acc);
        acc = 1;
      }
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                     smem_u32(&mbar))
                 : "memory");
  }
  // uniform verdict: the epilogue below contains a block barrier
  const bool ok = __syncthreads_and(mbar_wait(smem_u32(&mbar), 0)) != 0;
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  if (ok) {
    // TMEM -> shared memory (row r = 32 * warp + lane; the operand tiles are
    // dead once the MMAs have completed), then a coalesced read-modify-write
    // of A_ij with one 512-byte row per warp instruction.
    float* stg = reinterpret_cast<float*>(base);  // 128 x 129 floats
    const int r = 32 * warp + lane;
    for (int c0 = 0; c0 < kTile; c0 += 32) {
      uint32_t v[32];
      const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
          "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
            "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]),
            "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
            "=r"(v[30]), "=r"(v[31])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
      for (int q = 0; q < 32; ++q) stg[r * 129 + c0 + q] = __uint_as_float(v[q]);
    }
    __syncthreads();
    float* tile = mat + S.moff + (long long)(ti * kTile) * np + tj * kTile;
    // warp w owns rows w, w + 4, ...; eight rows in flight per batch
    for (int rb = warp; rb < kTile; rb += 8 * (kTcThreads / 32)) {
      float4 a[8];
#pragma unroll
      for (int u = 0; u < 8; ++u)
        a[u] = reinterpret_cast<const float4*>(tile + (long long)(rb + u * (kTcThreads / 32)) * np)[lane];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int rr = rb + u * (kTcThreads / 32);
        const float* sr = stg + rr * 129 + 4 * lane;
        a[u].x -= sr[0];
        a[u].y -= sr[1];
        a[u].z -= sr[2];
        a[u].w -= sr[3];
        reinterpret_cast<float4*>(tile + (long long)rr * np)[lane] = a[u];
      }
    }
  } else if (threadIdx.x == 0) {
    atomicOr(status + s, SFD_ST_TIMEOUT);
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    if (!ok) mbar_wait(smem_u32(&mbar), 0);  // give in-flight MMAs a second bounded chance
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTile));
  }
}

cudaError_t sfd_tc_configure() {
  return cudaFuncSetAttribute(k_gj_update_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              2 * kParts * kOpBytes + 1024);
}

cudaError_t sfd_launch_gj_update_tc(const SurfaceDesc* surf, int nsurf, int kb, int max_np, float* mat,
                                    const __nv_bfloat16* cparts, const __nv_bfloat16* rparts, long long part_stride,
                                    const long long* poff, unsigned int* status, cudaStream_t st) {
  const int t = max_np / kTile;
  k_gj_update_tc<<<dim3(t, t, nsurf), kTcThreads, 2 * kParts * kOpBytes + 1024, st>>>(surf, kb, mat, cparts, rparts,
                                                                                       part_stride, poff, status);
  return cudaPeekAtLastError();  // the caller's launch check reads and clears it
}
