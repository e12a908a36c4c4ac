// sfd_tc.cu -- tensor-core (tcgen05) trailing update of the blocked
// Gauss-Jordan preconditioner.
//
// Step kb of the in-place Gauss-Jordan inverse updates every 128 x 128 tile
// (i, j) outside block row / column K:
//     A_ij -= C_i R_j,   C_i = A_iK (128 x 128),  R_j = P A_Kj (128 x 128)
// a K = 128 GEMM per tile.  The panel kernel stores C and R^T split into three
// bf16 parts (x = hi + mid + lo: hi = bf16(x), mid = bf16(x - hi),
// lo = bf16(x - hi - mid); 24 significant bits, an FP32 value), K-major, each
// part a [rows x 128] array (rows of all surfaces concatenated).
//
// One persistent CTA per (tile column j, group of tile rows i), warp-specialised:
//   warp 0 (one lane)  TMA producer: R_j's three parts once (resident, 96 KB),
//                      then per tile the three parts of C_i in two K-halves of
//                      64, each 48 KB, through a two-stage ring;
//   warp 1 (one lane)  MMA issuer: per K-half 6 products x 4 tcgen05.mma
//                      (kind::f16, M = N = 128, K = 16), the products of order
//                      >= 2^-24 (hi.hi, hi.mid, mid.hi, hi.lo, mid.mid,
//                      lo.hi), FP32 accumulation in tensor memory; two
//                      accumulators (256 TMEM columns) so a tile's epilogue
//                      overlaps the next tile's MMAs;
//   warps 2-5          epilogue: tcgen05.ld of their 32-row quadrant, 32
//                      columns at a time, negated into a 128-byte-swizzled
//                      staging box (double-buffered per warp), and a TMA
//                      reduce-add (cp.reduce.async.bulk.tensor .add.f32) of
//                      the box into A_ij: the subtraction A_ij += (-C_i R_j)
//                      happens in L2, with no load of A_ij by the SM.
// The operand tiles arrive by cp.async.bulk.tensor (TMA) in the 128-byte
// swizzle the MMA descriptors read (8-row x 128-byte atoms, 16-byte chunk ^=
// row % 8); stage and accumulator hand-offs are mbarriers (TMA transaction
// counts, tcgen05.commit, epilogue arrivals).
// The result carries FP32-level error (~2^-24 relative per product), so the
// FP32 refinement corrections that follow stay small.
//
// Every wait is bounded: a wait that runs out sets SFD_ST_TIMEOUT in the
// surface status and an abort flag that every other wait of the CTA sees; the
// producer then waits (bounded) for its copies in flight, the MMA issuer for
// its MMAs, the tensor memory is freed and the CTA returns.
#include <cuda.h>
#include <cuda_bf16.h>

#include "sfd_engine.cuh"
#include "sfd_mbar.cuh"
#include "sfd_solve.cuh"

namespace {
using namespace sfd_async;

constexpr int kTile = 128;                       // M = N = K of one tile update
constexpr int kParts = 3;                        // bf16 parts per operand
constexpr int kHalfBytes = kTile * 128;          // one K-half of one part: 128 rows x 128 B (16 KB)
constexpr int kRBytes = kParts * 2 * kHalfBytes; // resident R_j: 3 parts x 2 K-halves (96 KB)
constexpr int kStageBytes = kParts * kHalfBytes; // one C stage: 3 parts of one K-half (48 KB)
constexpr int kStages = 2;
constexpr int kEpiWarps = 4;
constexpr int kThreads = 32 * (2 + kEpiWarps);   // producer, MMA issuer, 4 epilogue warps
constexpr int kBoxBytes = 32 * 32 * 4;           // epilogue staging box: 32 rows x 32 FP32 (128-byte rows)
constexpr int kSmemBytes = kRBytes + kStages * kStageBytes + kEpiWarps * 2 * kBoxBytes + 1024;
constexpr unsigned kSpinLimit = 1u << 22;

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

// Bounded wait that also gives up once another role of the CTA aborted.  A
// wait that runs out raises the abort flag and the timeout status bit.
__device__ __forceinline__ bool wait_or_abort(uint32_t mbar, uint32_t parity, volatile int* abort_flag,
                                              unsigned int* status) {
  for (unsigned it = 0; it < kSpinLimit; ++it) {
    if (mbar_try(mbar, parity)) return true;
    if ((it & 63u) == 63u && *abort_flag) return false;
  }
  *abort_flag = 1;
  atomicOr(status, SFD_ST_TIMEOUT);
  return false;
}
// Bounded wait used while winding down (ignores the abort flag).
__device__ __forceinline__ bool wait_bounded(uint32_t mbar, uint32_t parity) {
  for (unsigned it = 0; it < kSpinLimit; ++it)
    if (mbar_try(mbar, parity)) return true;
  return false;
}

// One K-half box (128 rows x 64 bf16) of part `part` at row `row`, K offset
// `k0` (0 or 64: k0 x 2 bytes is a multiple of 16).
__device__ __forceinline__ void tma_load_half(uint32_t sdst, const CUtensorMap* map, int k0, int row, int part,
                                              uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];\n" ::"r"(sdst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(k0), "r"(row), "r"(part), "r"(mbar)
      : "memory");
}
// dst[box at (x = column, y = row)] += src (FP32, 32 x 32 box, 128-byte swizzle)
__device__ __forceinline__ void tma_reduce_add(const CUtensorMap* map, int x, int y, uint32_t ssrc) {
  asm volatile(
      "cp.reduce.async.bulk.tensor.2d.global.shared::cta.add.tile.bulk_group [%0, {%1, %2}], [%3];\n" ::"l"(
          reinterpret_cast<uint64_t>(map)),
      "r"(x), "r"(y), "r"(ssrc)
      : "memory");
  asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
               : "memory");
}

}  // namespace

// Grid (tile columns, row groups, surfaces).  CTA (j, g, s) updates the tiles
// (i, j) of surface s for i in its row group, skipping block row and column
// kb (the SIMT kernel handles those).
__global__ void __launch_bounds__(kThreads, 1)
    k_gj_update_tc(const __grid_constant__ CUtensorMap map_c, const __grid_constant__ CUtensorMap map_r,
                   const CUtensorMap* map_out, const SurfaceDesc* surf, int kb, const long long* poff, int ngroups,
                   unsigned int* status) {
  const int s = blockIdx.z;
  const SurfaceDesc& S = surf[s];
  const int np = pad_n(S.n), nt = np / kTile, kt = kb;
  const int tj = blockIdx.x;
  if (kt >= nt || tj >= nt || tj == kt) return;
  const int rpg = (nt + ngroups - 1) / ngroups;
  const int i0 = blockIdx.y * rpg, i1 = min(nt, i0 + rpg);
  const int ntiles = (i1 - i0) - ((kt >= i0 && kt < i1) ? 1 : 0);
  if (ntiles <= 0) return;
  auto tile_row = [&](int t) {  // t-th row of the group, skipping kt
    const int i = i0 + t;
    return i >= kt ? i + (kt >= i0 ? 1 : 0) : i;
  };

  extern __shared__ uint8_t tc_smem_raw[];
  // operand tiles need 1024-byte alignment for the 128-byte swizzle
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~uintptr_t(1023));
  const uint32_t sR = smem_u32(base);
  const uint32_t sC = sR + kRBytes;  // stage q at sC + q * kStageBytes
  const uint32_t sStg = sC + kStages * kStageBytes;  // epilogue warp w, buffer b at sStg + (2 w + b) kBoxBytes
  __shared__ __align__(8) uint64_t bar_r, bar_full[kStages], bar_empty[kStages], bar_afull[2], bar_aempty[2];
  __shared__ uint32_t tmem_base_sh;
  __shared__ int abort_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned int* st = status + s;
  volatile int* abort_v = &abort_flag;

  if (threadIdx.x == 0) {
    abort_flag = 0;
    mbar_init(smem_u32(&bar_r), 1);
    for (int q = 0; q < kStages; ++q) {
      mbar_init(smem_u32(&bar_full[q]), 1);
      mbar_init(smem_u32(&bar_empty[q]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_u32(&bar_afull[b]), 1);
      mbar_init(smem_u32(&bar_aempty[b]), kEpiWarps);
    }
    mbar_init_fence();
  }
  // tensor memory: two FP32 accumulators of 128 columns (128 lanes = rows)
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_base_sh)),
                 "r"(2 * kTile));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_base_sh;
  const long long row_base = poff[s] / kTile;  // first row of this surface in the part arrays

  if (warp == 0) {
    // ------------------------------------------------------------ producer
    if (lane == 0) {
      const uint32_t br = smem_u32(&bar_r);
      mbar_expect_tx(br, kRBytes);
      for (int p = 0; p < kParts; ++p)
        for (int h = 0; h < 2; ++h)
          tma_load_half(sR + (p * 2 + h) * kHalfBytes, &map_r, 64 * h, (int)(row_base + (long long)tj * kTile), p,
                        br);
      int issued = 0;  // K-half chunks issued
      bool ok = true;
      for (int t = 0; t < ntiles && ok; ++t) {
        const int ti = tile_row(t);
        for (int h = 0; h < 2 && ok; ++h) {
          const int q = issued & 1, u = issued >> 1;
          ok = wait_or_abort(smem_u32(&bar_empty[q]), (uint32_t)((u & 1) ^ 1), abort_v, st);
          if (!ok) break;
          const uint32_t bf = smem_u32(&bar_full[q]);
          mbar_expect_tx(bf, kStageBytes);
          for (int p = 0; p < kParts; ++p)
            tma_load_half(sC + q * kStageBytes + p * kHalfBytes, &map_c, 64 * h,
                          (int)(row_base + (long long)ti * kTile), p, bf);
          ++issued;
        }
      }
      // wind down: the copies in flight land before the CTA may exit
      wait_bounded(br, 0);
      for (int c = max(0, issued - kStages); c < issued; ++c) wait_bounded(smem_u32(&bar_full[c & 1]), (c >> 1) & 1);
    }
  } else if (warp == 1) {
    // ---------------------------------------------------------- MMA issuer
    if (lane == 0) {
      bool ok = wait_or_abort(smem_u32(&bar_r), 0, abort_v, st);
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      // products with part-index sum <= 2: (hi,hi) (hi,mid) (mid,hi) (hi,lo) (mid,mid) (lo,hi)
      const int pa[6] = {0, 0, 1, 0, 1, 2}, pb[6] = {0, 1, 0, 2, 1, 0};
      int chunk = 0;
      int committed = 0;  // tiles whose accumulator commit was issued
      for (int t = 0; t < ntiles && ok; ++t) {
        const int b = t & 1, v = t >> 1;
        ok = wait_or_abort(smem_u32(&bar_aempty[b]), (uint32_t)((v & 1) ^ 1), abort_v, st);
        if (!ok) break;
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const uint32_t acc_tmem = tmem + (uint32_t)(b * kTile);
        for (int h = 0; h < 2 && ok; ++h) {
          const int q = chunk & 1, u = chunk >> 1;
          ok = wait_or_abort(smem_u32(&bar_full[q]), (uint32_t)(u & 1), abort_v, st);
          if (!ok) break;
          asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
          for (int p = 0; p < 6; ++p) {
            const uint32_t Ap = sC + q * kStageBytes + pa[p] * kHalfBytes;
            const uint32_t Bp = sR + (pb[p] * 2 + h) * kHalfBytes;
            for (int k4 = 0; k4 < 4; ++k4)  // 16 K-elements = 32 bytes inside the 128-byte atom
              mma_bf16(acc_tmem, make_sdesc(Ap + k4 * 32), make_sdesc(Bp + k4 * 32),
                       (h == 0 && p == 0 && k4 == 0) ? 0u : 1u);
          }
          mma_commit(smem_u32(&bar_empty[q]));  // the stage is free once these MMAs have read it
          ++chunk;
        }
        if (!ok) break;
        mma_commit(smem_u32(&bar_afull[b]));
        ++committed;
      }
      // wind down: the MMAs in flight complete before the tensor memory is freed
      if (committed > 0) wait_bounded(smem_u32(&bar_afull[(committed - 1) & 1]), ((committed - 1) >> 1) & 1);
      if (chunk > 0) wait_bounded(smem_u32(&bar_empty[(chunk - 1) & 1]), ((chunk - 1) >> 1) & 1);
    }
  } else {
    // ------------------------------------------------------------ epilogue
    const int quad = warp & 3;  // tcgen05.ld reaches TMEM lanes 32 (warp % 4) .. + 31
    const CUtensorMap* mo = map_out + s;
    if (lane == 0)
      asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;\n" ::"l"(reinterpret_cast<uint64_t>(mo))
                   : "memory");
    int nbox = 0;  // boxes issued by this warp (alternating staging buffers)
    for (int t = 0; t < ntiles; ++t) {
      const int b = t & 1, v = t >> 1;
      const bool ok = wait_or_abort(smem_u32(&bar_afull[b]), (uint32_t)(v & 1), abort_v, st);
      if (!__all_sync(0xffffffffu, ok)) break;
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const int row0 = tile_row(t) * kTile + 32 * quad;
      for (int c0 = 0; c0 < kTile; c0 += 32) {
        uint32_t r[32];
        const uint32_t taddr = tmem + ((uint32_t)(32 * quad) << 16) + (uint32_t)(b * kTile + c0);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
              "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
              "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
              "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
        if (c0 == kTile - 32) {
          // the accumulator has been read out: hand it back to the MMA issuer
          asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
          __syncwarp();
          if (lane == 0) mbar_arrive(smem_u32(&bar_aempty[b]));
        }
        // staging buffer: free once the reduce issued two boxes ago has read it
        if (lane == 0 && nbox >= 2) asm volatile("cp.async.bulk.wait_group.read 1;\n" ::: "memory");
        __syncwarp();
        const uint32_t box = sStg + (uint32_t)((2 * (warp - 2) + (nbox & 1)) * kBoxBytes);
        // row `lane` of the box, 16-byte chunk j at chunk position j ^ (lane % 8) (128-byte swizzle)
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const uint32_t a = box + (uint32_t)(lane * 128) + (uint32_t)((j ^ (lane & 7)) << 4);
          asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};\n" ::"r"(a), "f"(-__uint_as_float(r[4 * j])),
                       "f"(-__uint_as_float(r[4 * j + 1])), "f"(-__uint_as_float(r[4 * j + 2])),
                       "f"(-__uint_as_float(r[4 * j + 3]))
                       : "memory");
        }
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncwarp();
        if (lane == 0) tma_reduce_add(mo, tj * kTile + c0, row0, box);
        ++nbox;
      }
    }
    // the staging boxes stay valid until the reduces have read them
    if (lane == 0) asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory");
    __syncwarp();
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(2 * kTile));
  }
}

cudaError_t sfd_tc_configure() {
  return cudaFuncSetAttribute(k_gj_update_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
}

// Tensor maps of the bf16 parts (3 parts of `rows` K-major rows of 128 bf16,
// parts `part_stride` elements apart): boxes of 128 rows x 64 bf16 (one
// K-half, 128 bytes wide) in the 128-byte swizzle.
namespace {
using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                              const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
// cuTensorMapEncodeTiled from the driver, looked up once
cudaError_t get_encode(EncodeFn* out) {
  static EncodeFn encode = nullptr;
  if (!encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q{};
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess) return e;
    if (q != cudaDriverEntryPointSuccess || !fn) return cudaErrorNotSupported;
    encode = reinterpret_cast<EncodeFn>(fn);
  }
  *out = encode;
  return cudaSuccess;
}
}  // namespace

cudaError_t sfd_tc_make_map(void* map_out, const __nv_bfloat16* parts, long long rows, long long part_stride) {
  EncodeFn encode = nullptr;
  cudaError_t e = get_encode(&encode);
  if (e != cudaSuccess) return e;
  const cuuint64_t dims[3] = {(cuuint64_t)kTile, (cuuint64_t)rows, (cuuint64_t)kParts};
  const cuuint64_t strides[2] = {(cuuint64_t)kTile * 2, (cuuint64_t)part_stride * 2};  // bytes, dims 1 and 2
  const cuuint32_t box[3] = {64, (cuuint32_t)kTile, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = encode(reinterpret_cast<CUtensorMap*>(map_out), CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3,
                            const_cast<__nv_bfloat16*>(parts), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// Tensor map of one surface's FP32 matrix (np x np, row-major at `mat`):
// boxes of 32 rows x 32 columns (128-byte rows) in the 128-byte swizzle, the
// target of the update's reduce-adds.
cudaError_t sfd_tc_make_out_map(void* map_out, float* mat, int np) {
  EncodeFn encode = nullptr;
  cudaError_t e = get_encode(&encode);
  if (e != cudaSuccess) return e;
  const cuuint64_t dims[2] = {(cuuint64_t)np, (cuuint64_t)np};
  const cuuint64_t strides[1] = {(cuuint64_t)np * 4};
  const cuuint32_t box[2] = {32, 32};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = encode(reinterpret_cast<CUtensorMap*>(map_out), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, mat, dims,
                            strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

cudaError_t sfd_launch_gj_update_tc(const void* map_c, const void* map_r, const void* maps_out,
                                    const SurfaceDesc* surf, int nsurf, int kb, int max_np, int ngroups,
                                    const long long* poff, unsigned int* status, cudaStream_t st) {
  const int t = max_np / kTile;
  k_gj_update_tc<<<dim3(t, ngroups, nsurf), kThreads, kSmemBytes, st>>>(
      *reinterpret_cast<const CUtensorMap*>(map_c), *reinterpret_cast<const CUtensorMap*>(map_r),
      reinterpret_cast<const CUtensorMap*>(maps_out), surf, kb, poff, ngroups, status);
  return cudaPeekAtLastError();  // the caller's launch check reads and clears it
}
