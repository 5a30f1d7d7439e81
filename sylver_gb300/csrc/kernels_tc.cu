// Tensor-core Schur-complement update for FP32 fronts: C -= A B^T on the
// 5th-generation tensor cores (tcgen05, kind::f16 with BF16 operands) with
// the accumulator in tensor memory and operands staged by TMA.
//
// Accuracy: 3xBF16 with six products.  Each FP32 operand is split exactly
// into three BF16 parts x = x0 + x1 + x2 (x1 ~ 2^-8 x, x2 ~ 2^-16 x; the
// remainder is below 2^-24 x), and C -= A0 B0^T + A0 B1^T + A1 B0^T +
// A1 B1^T + A0 B2^T + A2 B0^T; the dropped products are below 2^-23 of the
// exact one, so each product is within FP32 rounding -- closer than a 4xTF32
// split (hi/lo of 11 bits each, 2^-22) at three quarters of its MMA time,
// since a BF16 MMA does twice the work of a TF32 one in the same time.  The
// tensor-core accumulator does not round to nearest, so its error over a long
// k range grows linearly (measured with TF32 operands: 16x an FP32 dot product
// at k = 4096); the accumulator is therefore drained into FP32 registers after
// every 64-wide k chunk and the chunks are summed there, which brings the
// update to FP32 accuracy and lets FP64 refinement converge as for SIMT FP32
// factors.
//
// Operand layout: the MMAs read K-major shared-memory tiles, so A and B come
// from a transposed copy of the rows of L below the eliminated columns
// ("panel rows", one row per front row, k contiguous, zero-padded to a
// multiple of 64) stacked for all fronts of a launch with a fixed pitch, one
// plane per BF16 part; one 2D tensor map per plane covers it.  TMA boxes are
// 64 (k) x 128 (rows) BF16 with 128-byte swizzle, matching the tcgen05
// K-major SWIZZLE_128B canonical layout.
//
// A persistent CTA per SM walks the launch's 128 x 128 tiles (10 warps): a TMA
// producer, an MMA issuer (24 MMAs per 64-wide k chunk; tcgen05.commit
// releases a stage and signals an accumulator) and eight epilogue warps that
// tcgen05.ld their 32 TMEM lanes after every chunk and subtract it from the
// C values they hold in registers while the next chunks' MMAs run in the
// other three accumulators of a four-deep TMEM ring; C is written once per
// tile.
// Every mbarrier wait is bounded: on timeout the CTA records an error bit,
// skips the epilogue, waits (bounded) for its own copies and frees TMEM.
#include <cuda.h>
#include <cudaTypedefs.h>

#include "device.hpp"
#include "tc.hpp"

namespace sylver_gb300 {

namespace {

constexpr int TC_M = 128, TC_N = 128, TC_KC = TC_KCHUNK;  // tile rows, cols, k per stage
constexpr int TC_STAGES = 2;
constexpr int TC_PLANES = 3;                        // BF16 parts of an operand
constexpr int TILE_BYTES = TC_M * TC_KC * 2;        // 16 KiB per operand tile
constexpr int STAGE_BYTES = 2 * TC_PLANES * TILE_BYTES;  // A0 A1 A2 B0 B1 B2
constexpr long WAIT_LIMIT = 1L << 24;               // try_wait polls before giving up

__device__ __forceinline__ uint32_t su32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(b)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(su32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// bounded wait (poll count and one second of wall time); false, with the
// error bit set, on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity, unsigned* err) {
  const uint64_t t0 = global_ns();
  for (long it = 0; it < WAIT_LIMIT; ++it) {
    if (mbar_try(b, parity)) return true;
    if ((it & 255) == 255 && global_ns() - t0 > 1000000000ull) break;
  }
  atomicOr(err, ST_TIMEOUT);
  return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(su32(dst)),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(su32(bar))
      : "memory");
}

// K-major, 128-byte swizzle shared-memory matrix descriptor (tcgen05 format:
// start >> 4 in bits 0-13, leading byte offset >> 4 in 16-29 (unused for a
// swizzled K-major tile), stride byte offset >> 4 in 32-45 = 1024 B between
// 8-row groups, version 1 in bits 46-47, swizzle mode 2 (128 B) in 61-63).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// instruction descriptor (kind::f16): D f32 (bits 4-5 = 1), A and B bf16
// (bits 7-9 and 10-12 = 1), both K-major, N >> 3 in bits 17-22, M >> 4 in
// bits 24-28
__host__ __device__ constexpr uint32_t bf16_idesc() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TC_N >> 3) << 17) |
         ((uint32_t)(TC_M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t ad, uint64_t bd,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          su32(bar))
      : "memory");
}

template <int N>
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[N]);

template <>
__device__ __forceinline__ void tmem_ld32<32>(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

// ---------------------------------------------------------------------------

constexpr int TC_EPI_WARP0 = 2;                  // warps 2..9 run the epilogue
constexpr int TC_EPI_WARPS = 8;                  // two per TMEM lane quarter
constexpr int TC_EPI_COLS = TC_N / 2;            // columns per epilogue thread
constexpr int TC_THREADS = 32 * (TC_EPI_WARP0 + TC_EPI_WARPS);
constexpr int TC_NACC = 4;                       // accumulators in the TMEM ring
constexpr int TC_TMEM_COLS = TC_NACC * TC_N;     // all 512 TMEM columns

// arrive on an mbarrier (one arrival)
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(b)) : "memory");
}

// bounded wait that also gives up once another role has aborted
__device__ __forceinline__ bool mbar_wait_or_abort(uint64_t* b, uint32_t parity, unsigned* err,
                                                   volatile int* abort_flag) {
  const uint64_t t0 = global_ns();
  for (long it = 0; it < WAIT_LIMIT; ++it) {
    if (mbar_try(b, parity)) return true;
    if ((it & 255) == 255) {
      if (*abort_flag) return false;
      if (global_ns() - t0 > 1000000000ull) break;
    }
  }
  atomicOr(err, ST_TIMEOUT);
  *abort_flag = 1;
  return false;
}

// Persistent: CTA b processes tiles b, b + gridDim.x, ...
//   warp 0 lane 0 : TMA producer over a TC_STAGES ring shared by all tiles,
//   warp 1 lane 0 : MMA issuer; k chunk i (counted over all tiles of the
//                   CTA) accumulates in TMEM columns [(i % 4) * 128, +128) so
//                   the epilogue's read of chunk i overlaps the MMAs of the
//                   next three chunks,
//   warps 2..9    : epilogue; each thread owns half a row of the tile, loads
//                   its 64 C values before the first chunk is ready,
//                   subtracts every chunk, releases the accumulator after
//                   each, and stores C after the tile's last chunk.
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_update_tc(const __grid_constant__ CUtensorMap map0,
                const __grid_constant__ CUtensorMap map1,
                const __grid_constant__ CUtensorMap map2, float* __restrict__ arena,
                const TcTask* __restrict__ tasks, int ntask, unsigned* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1 KiB alignment for the swizzled tiles
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  __shared__ uint64_t full[TC_STAGES], empty[TC_STAGES], acc_full[TC_NACC], acc_empty[TC_NACC],
      done;
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  volatile int* abortp = &abort_flag;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < TC_STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int a = 0; a < TC_NACC; ++a) {
      mbar_init(&acc_full[a], 1);
      mbar_init(&acc_empty[a], TC_EPI_WARPS);  // one arrival per epilogue warp
    }
    mbar_init(&done, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     su32(&tmem_slot)),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;

  int issued = 0;  // TMA chunks issued by the producer
  if (warp == 0) {
    if (lane == 0) {
      int g = 0;
      for (int ti = blockIdx.x; ti < ntask && !*abortp; ti += gridDim.x) {
        const TcTask t = tasks[ti];
        bool ok = true;
        for (int kc = 0; kc < t.nk; ++kc, ++g) {
          const int s = g % TC_STAGES;
          if (g >= TC_STAGES &&
              !mbar_wait_or_abort(&empty[s], ((g / TC_STAGES) - 1) & 1, err, abortp)) {
            ok = false;
            break;
          }
          unsigned char* st = smem + s * STAGE_BYTES;
          mbar_expect_tx(&full[s], STAGE_BYTES);
          const int x = (t.kc0 + kc) * TC_KC;
          tma_load_2d(st + 0 * TILE_BYTES, &map0, x, t.a_row, &full[s]);
          tma_load_2d(st + 1 * TILE_BYTES, &map1, x, t.a_row, &full[s]);
          tma_load_2d(st + 2 * TILE_BYTES, &map2, x, t.a_row, &full[s]);
          tma_load_2d(st + 3 * TILE_BYTES, &map0, x, t.b_row, &full[s]);
          tma_load_2d(st + 4 * TILE_BYTES, &map1, x, t.b_row, &full[s]);
          tma_load_2d(st + 5 * TILE_BYTES, &map2, x, t.b_row, &full[s]);
          issued = g + 1;
        }
        if (!ok) break;
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = bf16_idesc();
      int g = 0, it = 0;  // it counts accumulator uses (one per k chunk)
      bool ok = true;
      for (int ti = blockIdx.x; ti < ntask && ok; ti += gridDim.x) {
        const int nk = tasks[ti].nk;
        for (int kc = 0; kc < nk; ++kc, ++g, ++it) {
          const int a = it % TC_NACC;
          // accumulator a was last used by chunk it - TC_NACC: wait until the
          // epilogue has read it
          if (it >= TC_NACC &&
              !mbar_wait_or_abort(&acc_empty[a], ((it / TC_NACC) - 1) & 1, err, abortp)) {
            ok = false;
            break;
          }
          const int s = g % TC_STAGES;
          if (!mbar_wait_or_abort(&full[s], (g / TC_STAGES) & 1, err, abortp)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t d = tmem + (uint32_t)(a * TC_N);
          unsigned char* st = smem + s * STAGE_BYTES;
          const uint64_t a0 = sw128_desc(su32(st + 0 * TILE_BYTES));
          const uint64_t a1 = sw128_desc(su32(st + 1 * TILE_BYTES));
          const uint64_t a2 = sw128_desc(su32(st + 2 * TILE_BYTES));
          const uint64_t b0 = sw128_desc(su32(st + 3 * TILE_BYTES));
          const uint64_t b1 = sw128_desc(su32(st + 4 * TILE_BYTES));
          const uint64_t b2 = sw128_desc(su32(st + 5 * TILE_BYTES));
#pragma unroll
          for (int kk = 0; kk < TC_KC / 16; ++kk) {
            // 16 bf16 = 32 bytes further along k inside the swizzled row;
            // small products first
            const uint64_t adv = (uint64_t)((kk * 32) >> 4);
            mma_bf16(d, a2 + adv, b0 + adv, idesc, kk > 0 ? 1u : 0u);
            mma_bf16(d, a0 + adv, b2 + adv, idesc, 1u);
            mma_bf16(d, a1 + adv, b1 + adv, idesc, 1u);
            mma_bf16(d, a1 + adv, b0 + adv, idesc, 1u);
            mma_bf16(d, a0 + adv, b1 + adv, idesc, 1u);
            mma_bf16(d, a0 + adv, b0 + adv, idesc, 1u);
          }
          mma_commit(&empty[s]);
          mma_commit(&acc_full[a]);
        }
      }
      // every MMA issued so far has completed once `done` fires
      mma_commit(&done);
    }
  } else {
    // TMEM lanes [32q, 32q + 32) are this warp's; it owns columns
    // [h * 64, h * 64 + 64) of each tile.  The tensor cores accumulate one
    // 32-wide k chunk at a time; the running sum over chunks is kept in
    // registers and added with IEEE FP32 arithmetic, so the error of a long
    // update grows like that of an FP32 dot product, not linearly in k.
    const int q = warp & 3, h = (warp - TC_EPI_WARP0) >> 2;
    int it = 0;
    bool ok = true;
    for (int ti = blockIdx.x; ti < ntask && ok; ti += gridDim.x) {
      const TcTask t = tasks[ti];
      const int row = t.row0 + q * 32 + lane;
      const int c0 = t.col0 + h * TC_EPI_COLS;
      // columns [c0, cend) of this row are updated (lower triangle, in range)
      const int cend = row < t.rowEnd ? min(t.colEnd, row + 1) : c0;
      const int64_t ldc = t.ldc;
      const float* src = arena + t.c_off + row + (int64_t)c0 * ldc;
      float cv[TC_EPI_COLS];
#pragma unroll
      for (int j = 0; j < TC_EPI_COLS; ++j) {
        cv[j] = c0 + j < cend ? *src : 0.f;
        src += ldc;
      }
      for (int kc = 0; kc < t.nk; ++kc, ++it) {
        const int a = it % TC_NACC;
        // warp-uniform wait: tcgen05.ld below is a warp-collective instruction
        int ready = 0;
        if (lane == 0) ready = mbar_wait_or_abort(&acc_full[a], (it / TC_NACC) & 1, err, abortp);
        ready = __shfl_sync(0xffffffffu, ready, 0);
        if (!ready) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
        for (int c = 0; c < TC_EPI_COLS / 32; ++c) {
          float v[32];
          tmem_ld32<32>(tmem + ((uint32_t)(q * 32) << 16) +
                            (uint32_t)(a * TC_N + h * TC_EPI_COLS + c * 32),
                        v);
#pragma unroll
          for (int j = 0; j < 32; ++j) cv[c * 32 + j] -= v[j];
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(&acc_empty[a]);
      }
      if (!ok) break;
      // recompute the store addresses and bounds here (opaque copies):
      // reusing the load-side ones would keep 64 of each live across the loop
      float* dst = arena + t.c_off + row + (int64_t)c0 * ldc;
      int cst = c0, cen = cend;
      asm volatile("mov.b64 %0, %0;" : "+l"(dst));
      asm volatile("mov.b32 %0, %0;" : "+r"(cst));
      asm volatile("mov.b32 %0, %0;" : "+r"(cen));
#pragma unroll
      for (int j = 0; j < TC_EPI_COLS; ++j) {
        if (cst + j < cen) *dst = cv[j];
        dst += ldc;
      }
    }
  }
  __syncthreads();
  // all MMAs this CTA issued have drained once `done` fires; wait for it even
  // after a failure, before TMEM is freed
  mbar_wait(&done, 0, err);
  // copies still in flight after a failure: wait (bounded) for the last one
  // issued on each stage before the shared memory they target goes away
  if (*abortp && warp == 0 && lane == 0) {
    for (int g = issued - 1; g >= 0 && g >= issued - TC_STAGES; --g)
      mbar_wait(&full[g % TC_STAGES], (g / TC_STAGES) & 1, err);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TC_TMEM_COLS)
                 : "memory");
}

// Transposed, 3xBF16-split copy of rows [n, m) x cols [c0, c0 + K) of one
// front into the stacked panel planes: plane q at planes + q * pstride,
// element (base + i - n) * pitch + k; columns [K, pitch) are zero.  A 32 x 32
// tile per CTA (32 x 8 threads) goes through shared memory, so both the
// column reads from the front and the row writes to the planes are
// coalesced.
__global__ void __launch_bounds__(256) k_split_t(const float* __restrict__ arena,
                                                 const TcSplit* __restrict__ sp,
                                                 uint16_t* __restrict__ planes,
                                                 int64_t pstride, int pitch) {
  __shared__ float tile[32][33];  // tile[k][i]
  const TcSplit t = sp[blockIdx.z];
  const int rows = t.m - t.n;
  const int i0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  if (i0 >= rows) return;  // uniform over the CTA
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int kk = ty; kk < 32; kk += 8) {
    const int k = k0 + kk, i = i0 + tx;
    tile[kk][tx] = (k < t.K && i < rows)
                       ? arena[t.off + (int64_t)(t.c0 + k) * t.ld + t.n + i] : 0.f;
  }
  __syncthreads();
  for (int ii = ty; ii < 32; ii += 8) {
    const int i = i0 + ii;
    if (i >= rows) break;
    uint16_t b0, b1, b2;
    bf16x3_split(tile[tx][ii], b0, b1, b2);
    const int64_t o = (int64_t)(t.base + i) * pitch + k0 + tx;
    planes[o] = b0;
    planes[pstride + o] = b1;
    planes[2 * pstride + o] = b2;
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    SG_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !p) throw CudaError("cuTensorMapEncodeTiled missing");
    fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  }
  return fn;
}

}  // namespace

size_t tc_smem_bytes() { return (size_t)TC_STAGES * STAGE_BYTES + 1024; }

static int g_num_sms = 0;

void prepare_tc_kernels() {
  SG_CUDA(cudaFuncSetAttribute(k_update_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)tc_smem_bytes()));
  int dev = 0;
  SG_CUDA(cudaGetDevice(&dev));
  SG_CUDA(cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev));
}

void make_panel_map(CUtensorMap* map, const uint16_t* base, int64_t rows, int pitch) {
  // 2D: x = k (contiguous, pitch BF16 elements), y = stacked panel row
  cuuint64_t dims[2] = {(cuuint64_t)pitch, (cuuint64_t)std::max<int64_t>(rows, 1)};
  cuuint64_t strides[1] = {(cuuint64_t)pitch * sizeof(uint16_t)};
  cuuint32_t box[2] = {(cuuint32_t)TC_KC, (cuuint32_t)TC_M};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = encode_fn()(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)base, dims, strides,
                           box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw CudaError("cuTensorMapEncodeTiled failed");
}

void launch_split_t(const float* arena, const TcSplit* sp, int nsplit, int64_t max_rows,
                    uint16_t* planes, int64_t pstride, int pitch, cudaStream_t s) {
  if (nsplit <= 0 || max_rows <= 0) return;
  // pitch is a multiple of 64: every k of a tile lies inside the row
  dim3 grid((unsigned)((max_rows + 31) / 32), (unsigned)(pitch / 32), (unsigned)nsplit);
  k_split_t<<<grid, 256, 0, s>>>(arena, sp, planes, pstride, pitch);
}

void launch_update_tc(const CUtensorMap* maps, float* arena, const TcTask* t, int ntask,
                      unsigned* err, cudaStream_t s) {
  if (ntask <= 0) return;
  // one persistent CTA per SM (the shared-memory ring admits one per SM)
  const int grid = std::min(ntask, g_num_sms > 0 ? g_num_sms : 148);
  k_update_tc<<<grid, TC_THREADS, tc_smem_bytes(), s>>>(maps[0], maps[1], maps[2], arena, t,
                                                         ntask, err);
}

}  // namespace sylver_gb300
