// Cholesky-side kernels of the level schedule: A->front initialisation,
// extend-add of contribution blocks, small fronts factorised whole in shared
// memory, panel Cholesky + triangular solve, and the tile update
// C -= A_rows A_cols^T used for both the trailing fully-summed update and the
// contribution-block (Schur complement) update.
//
// Reference behaviour replaced:
//   init_a_block / init_node         src/kernels/assemble.hxx:162-214
//   assemble_block / _contrib_block  src/kernels/assemble.hxx:231-286, :344-425
//   factorize_diag_block + solve_block + update_block + update_diag_block
//                                     src/kernels/factor.hxx:56-260,
//                                     src/factor.hxx:19-148
#include <type_traits>

#include "device.hpp"
#include "tile_update.cuh"

namespace sylver_gb300 {

namespace {

template <typename T> __device__ __forceinline__ void atomic_add(T* p, T v) { atomicAdd(p, v); }

// ---------------------------------------------------------------------------
// Lower triangles of the fronts set to zero before assembly, one CTA per task
// (a range of columns); warps take columns, lanes run down the rows.
template <typename T>
__global__ void __launch_bounds__(256) k_zero_lower(T* __restrict__ arena,
                                                    const ZeroTask* __restrict__ tasks) {
  const ZeroTask t = tasks[blockIdx.x];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int j = t.j0 + warp; j < t.j1; j += 8) {
    T* col = arena + t.off + (int64_t)j * t.ld;
    for (int i = j + lane; i < t.m; i += 32) col[i] = T(0);
  }
}

// Whole spans of the arena <- 0 (front blocks placed where contribution
// blocks were given back), 16-byte stores; one CTA per span.
template <typename T>
__global__ void __launch_bounds__(256) k_zero_spans(T* __restrict__ arena,
                                                    const ZeroSpan* __restrict__ spans) {
  const ZeroSpan z = spans[blockIdx.x];
  float4* p = reinterpret_cast<float4*>(arena + z.off);
  const int64_t n4 = z.len * (int64_t)sizeof(T) / 16;
  for (int64_t i = threadIdx.x; i < n4; i += 256) p[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// Copies of whole spans (a front's factor columns into the compact factor
// store), 16-byte loads and stores; one CTA per span.
template <typename T>
__global__ void __launch_bounds__(256) k_copy_spans(T* __restrict__ dst, const T* __restrict__ src,
                                                    const CopySpan* __restrict__ spans) {
  const CopySpan c = spans[blockIdx.x];
  const float4* s4 = reinterpret_cast<const float4*>(src + c.src);
  float4* d4 = reinterpret_cast<float4*>(dst + c.dst);
  const int64_t n4 = c.len * (int64_t)sizeof(T) / 16;
  for (int64_t i = threadIdx.x; i < n4; i += 256) d4[i] = s4[i];
}

// arena[dst[k]] (+)= val[src[k]]  -- assembly of original entries.
template <typename T>
__global__ void k_init_a(T* __restrict__ arena, const double* __restrict__ val,
                         const int64_t* __restrict__ src, const int64_t* __restrict__ dst,
                         int64_t count, bool atomic) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (; k < count; k += stride) {
    T v = (T)val[src[k]];
    if (atomic) atomic_add(arena + dst[k], v);
    else arena[dst[k]] = v;
  }
}

// One warp per (child, CB column): parent(map[i], map[j]) += cb(i, j), i >= j.
// Two children of one parent may hit the same parent entry: with `atomic`
// the launch may hold several children of a parent; without it the caller
// gives each launch at most one child per parent (children in a fixed order
// across launches), which makes the sums deterministic.  The column is read
// in 16-byte pieces: front storage starts on a 64-element boundary with a
// leading dimension divisible by 4, so the pieces are aligned from the
// first aligned row on (the rows before it, at most three, are read singly),
// and a piece never reaches past the column's padded length.
template <typename T>
__device__ __forceinline__ void ea_column(T* __restrict__ arena, const ChildDesc& c,
                                          const int* __restrict__ maps, int j, int lane,
                                          bool atomic) {
  constexpr int V = 16 / sizeof(T);
  using Vec = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
  const int* map = maps + c.map_off;
  const int pj = map[j];
  const int64_t s0 = c.cb_off + (int64_t)j * c.ld_c;  // element index of cb(0, j)
  const T* src = arena + s0;
  T* dst = arena + c.p_off;
  auto addr = [&](int pi) {
    const int r = max(pi, pj), cc = min(pi, pj);
    return dst + (int64_t)cc * c.ld_p + r;
  };
  const int mis = (int)((s0 + j) % V);
  const int ia = j + (mis ? V - mis : 0);  // first row >= j on a 16-byte boundary
  if (j + lane < min(ia, c.mc)) {
    T* d = addr(map[j + lane]);
    if (atomic) atomic_add(d, src[j + lane]);
    else *d += src[j + lane];
  }
  // EB pieces per lane per round: every load of the round (the column, its
  // map entries, then the parent entries) is issued before the first store
  constexpr int EB = 2;
  for (int i0 = ia + lane * V; i0 < c.mc; i0 += 32 * V * EB) {
    T e[EB][V];
    int pi[EB][V];
#pragma unroll
    for (int b = 0; b < EB; ++b) {
      const int i = i0 + b * 32 * V;
      if (i < c.mc) {
        const Vec v = *reinterpret_cast<const Vec*>(src + i);
        if constexpr (V == 4) {
          e[b][0] = v.x; e[b][1] = v.y; e[b][2] = v.z; e[b][3] = v.w;
        } else {
          e[b][0] = v.x; e[b][1] = v.y;
        }
      }
#pragma unroll
      for (int u = 0; u < V; ++u) pi[b][u] = (i + u < c.mc) ? map[i + u] : -1;
    }
    if (atomic) {
#pragma unroll
      for (int b = 0; b < EB; ++b)
#pragma unroll
        for (int u = 0; u < V; ++u)
          if (pi[b][u] >= 0) atomic_add(addr(pi[b][u]), e[b][u]);
    } else {
      T old[EB][V];
#pragma unroll
      for (int b = 0; b < EB; ++b)
#pragma unroll
        for (int u = 0; u < V; ++u) old[b][u] = pi[b][u] >= 0 ? *addr(pi[b][u]) : T(0);
#pragma unroll
      for (int b = 0; b < EB; ++b)
#pragma unroll
        for (int u = 0; u < V; ++u)
          if (pi[b][u] >= 0) *addr(pi[b][u]) = old[b][u] + e[b][u];
    }
  }
}

template <typename T>
__global__ void k_extend_add(T* __restrict__ arena, const ChildDesc* __restrict__ cd,
                             const EaItem* __restrict__ items, const int* __restrict__ maps,
                             int nitems, bool atomic) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp >= nitems) return;
  const EaItem it = items[warp];
  ea_column<T>(arena, cd[it.child], maps, it.col, threadIdx.x & 31, atomic);
}

// One warp per parent column: the CB columns of the front's children that
// map to it (group g: items [grp[g], grp[g + 1]), in child order) are added
// one after another, so every parent entry receives its children's sums in a
// fixed order without atomics.  Needs maps that keep row order (a child
// column then lands in one parent column).
template <typename T>
__global__ void k_extend_add_grouped(T* __restrict__ arena, const ChildDesc* __restrict__ cd,
                                     const EaItem* __restrict__ items,
                                     const int* __restrict__ grp, const int* __restrict__ maps,
                                     int ngroups) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp >= ngroups) return;
  const int lane = threadIdx.x & 31;
  for (int q = grp[warp]; q < grp[warp + 1]; ++q) {
    const EaItem it = items[q];
    ea_column<T>(arena, cd[it.child], maps, it.col, lane, false);
    __syncwarp();  // this column's additions land before the next child's
  }
}

// Assembly of a level's fronts in one pass (child row maps that keep row
// order): one warp per front column builds rows [j, m) of column j in chunks
// of R rows in shared memory — zero, the column's original entries, then each
// child CB column that lands there, in child order — and stores every chunk
// once.  The front needs no zeroing beforehand and its entries no read-modify-
// write, and every entry gets the sum of zeroing + k_init_a + the grouped
// extend-add: (0 + a) then the children in order, bit for bit.  A child
// column is read from its first row on in rounds of 32 x U rows; its rows
// land in increasing parent rows, so the rows of a round that fall inside the
// chunk are a prefix of it and the next chunk resumes after them.  Each
// column's metadata is loaded once, spread over the lanes: lane q holds item
// q's child column (next row, rows, map, source) and the column's first 32
// original entries sit one per lane.
template <typename T>
__global__ void __launch_bounds__(256) k_assemble(T* __restrict__ arena,
                                                  const double* __restrict__ val,
                                                  const AsmTask* __restrict__ tasks,
                                                  const int* __restrict__ acp,
                                                  const int* __restrict__ arow,
                                                  const int64_t* __restrict__ asrc,
                                                  const int* __restrict__ gptr,
                                                  const EaItem* __restrict__ items,
                                                  const ChildDesc* __restrict__ cd,
                                                  const int* __restrict__ maps) {
  constexpr int R = 4096 / (int)sizeof(T);
  constexpr int U = 8;
  constexpr unsigned FULL = 0xffffffffu;
  __shared__ T sbuf[8][R];
  const AsmTask t = tasks[blockIdx.x];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T* buf = sbuf[warp];
  for (int j = t.j0 + warp; j < t.j1; j += 8) {
    T* col = arena + t.off + (int64_t)j * t.ld;
    const int cj = t.cbase + j;
    const int a0 = acp[cj], a1 = acp[cj + 1], g0 = gptr[cj], ng = gptr[cj + 1] - g0;
    int cur = 0, cmc = 0;
    unsigned long long cmap = 0, csrc = 0;
    if (lane < ng) {
      const EaItem it = items[g0 + lane];
      const ChildDesc c = cd[it.child];
      cur = it.col;
      cmc = c.mc;
      cmap = (unsigned long long)(maps + c.map_off);
      csrc = (unsigned long long)(arena + c.cb_off + (int64_t)it.col * c.ld_c);
    }
    int ar = -1;
    T av = T(0);
    if (a0 + lane < a1) {
      ar = arow[a0 + lane];
      av = (T)val[asrc[a0 + lane]];
    }
    for (int r0 = j; r0 < t.m; r0 += R) {
      const int nr = min(R, t.m - r0), r1 = r0 + nr;
      for (int i = lane; i < nr; i += 32) buf[i] = T(0);
      __syncwarp();
      if (ar >= r0 && ar < r1) buf[ar - r0] = av;
      for (int e = a0 + 32 + lane; e < a1; e += 32) {
        const int r = arow[e];
        if (r >= r0 && r < r1) buf[r - r0] = (T)val[asrc[e]];
      }
      __syncwarp();
      for (int q = 0; q < ng; ++q) {
        const int mc = __shfl_sync(FULL, cmc, q);
        const int* map = reinterpret_cast<const int*>(__shfl_sync(FULL, cmap, q));
        const T* src = reinterpret_cast<const T*>(__shfl_sync(FULL, csrc, q));
        int i = __shfl_sync(FULL, cur, q);
        for (;;) {
          int pr[U];
          T v[U];
#pragma unroll
          for (int u = 0; u < U; ++u) {
            const int ii = i + u * 32 + lane;
            pr[u] = ii < mc ? map[ii] : r1;
            v[u] = ii < mc ? src[ii] : T(0);
          }
          int cnt = 0;
#pragma unroll
          for (int u = 0; u < U; ++u) {
            const bool ok = pr[u] < r1;
            if (ok) buf[pr[u] - r0] += v[u];
            cnt += __popc(__ballot_sync(FULL, ok));
          }
          i += cnt;
          if (cnt < U * 32) break;
        }
        if (lane == q) cur = i;
        __syncwarp();  // this child's additions land before the next one's
      }
      for (int i = lane; i < nr; i += 32) col[r0 + i] = buf[i];
      __syncwarp();
    }
  }
}

// ---------------------------------------------------------------------------
// Whole-front partial Cholesky in shared memory (m <= SMALL_M): eliminate the
// first n columns and update the contribution block in place.
template <typename T>
__global__ void __launch_bounds__(256) k_small_chol(T* __restrict__ arena,
                                                    const SmallTask* __restrict__ tasks,
                                                    unsigned* status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s = reinterpret_cast<T*>(smem_raw);
  SmallTask t = tasks[blockIdx.x];
  const int m = t.m, n = t.n, lds = m + 1;
  T* a = arena + t.off;
  for (int idx = threadIdx.x; idx < m * m; idx += blockDim.x) {
    int i = idx % m, j = idx / m;
    if (i >= j) s[j * lds + i] = a[(int64_t)j * t.ld + i];
  }
  __syncthreads();
  __shared__ T dkk;
  for (int k = 0; k < n; ++k) {
    if (threadIdx.x == 0) {
      T d = s[k * lds + k];
      if (!(d > T(0))) {
        atomicOr(status, ST_NOT_POSDEF);
        d = T(1);
      }
      d = sqrt(d);
      s[k * lds + k] = d;
      dkk = T(1) / d;
    }
    __syncthreads();
    T inv = dkk;
    for (int i = k + 1 + threadIdx.x; i < m; i += blockDim.x) s[k * lds + i] *= inv;
    __syncthreads();
    const int w = m - k - 1;
    for (int idx = threadIdx.x; idx < w * w; idx += blockDim.x) {
      int i = k + 1 + idx % w, j = k + 1 + idx / w;
      if (i >= j) s[j * lds + i] -= s[k * lds + i] * s[k * lds + j];
    }
    __syncthreads();
  }
  for (int idx = threadIdx.x; idx < m * m; idx += blockDim.x) {
    int i = idx % m, j = idx / m;
    if (i >= j) a[(int64_t)j * t.ld + i] = s[j * lds + i];
  }
}

// ---------------------------------------------------------------------------
// Panel step, part 1: Cholesky of the w x w diagonal block at (k0, k0), one
// CTA of four warps per front, in shared memory: warp q updates the trailing
// columns j = q (mod 4), lanes run down the rows.
template <typename T, int NB>
__global__ void __launch_bounds__(128) k_diag_chol(T* __restrict__ arena,
                                                   const PanelTask* __restrict__ tasks,
                                                   unsigned* status) {
  __shared__ T D[NB][NB + 1];  // D[j][i] = A(i, j)
  const PanelTask t = tasks[blockIdx.x];
  T* a = arena + t.off;
  const int ld = t.ld, k0 = t.k0, w = t.w, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
#pragma unroll 4
  for (int e = tid; e < NB * NB; e += 128) {
    int i = e % NB, j = e / NB;
    if (i < w && j < w && i >= j) D[j][i] = a[(int64_t)(k0 + j) * ld + k0 + i];
  }
  __syncthreads();
  for (int k = 0; k < w; ++k) {
    T d = D[k][k];
    if (!(d > T(0))) {
      if (tid == 0) atomicOr(status, ST_NOT_POSDEF);
      d = T(1);
    }
    const T inv = T(1) / sqrt(d);
    // column k below the diagonal, scaled into registers; row k+1.. by lanes
    for (int j = k + 1 + warp; j < w; j += 4) {
      const T ljk = D[k][j] * inv;
      for (int i = j + lane; i < w; i += 32) D[j][i] -= D[k][i] * inv * ljk;
    }
    __syncthreads();
    if (tid == 0) D[k][k] = sqrt(d);
    for (int i = k + 1 + tid; i < w; i += 128) D[k][i] *= inv;
    __syncthreads();
  }
#pragma unroll 4
  for (int e = tid; e < NB * NB; e += 128) {
    int i = e % NB, j = e / NB;
    if (i < w && j < w && i >= j) a[(int64_t)(k0 + j) * ld + k0 + i] = D[j][i];
  }
}

// Panel step, part 2: rows [r0, r1) below the diagonal block solve
// L_r = A_r L_kk^-T against the factor written by k_diag_chol.
template <typename T, int NB, int RT>
__global__ void __launch_bounds__(RT) k_panel_trsm(T* __restrict__ arena,
                                                   const PanelTask* __restrict__ tasks) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* D = reinterpret_cast<T*>(smem_raw);  // NB x (NB+1), column-major
  T* R = D + NB * (NB + 1);               // NB x (RT+1): R[k*(RT+1) + row]
  __shared__ T dinv[NB];
  const PanelTask t = tasks[blockIdx.x];
  T* a = arena + t.off;
  const int ld = t.ld, k0 = t.k0, w = t.w;
  const int tid = threadIdx.x;
  constexpr int LDD = NB + 1, LDR = RT + 1;
  for (int idx = tid; idx < w * w; idx += RT) {
    int i = idx % w, j = idx / w;
    D[j * LDD + i] = (i >= j) ? a[(int64_t)(k0 + j) * ld + k0 + i] : T(0);
  }
  const int r = t.r0 + tid;
  const bool has_row = r < t.r1;
  if (has_row) {
#pragma unroll 16
    for (int k = 0; k < NB; ++k)
      if (k < w) R[k * LDR + tid] = a[(int64_t)(k0 + k) * ld + r];
  }
  __syncthreads();
  if (tid < w) dinv[tid] = T(1) / D[tid * LDD + tid];
  __syncthreads();
  if (has_row) {
    // x L_kk^T = a_r  (forward substitution along the row)
    for (int j = 0; j < w; ++j) {
      T x = R[j * LDR + tid] * dinv[j];
      R[j * LDR + tid] = x;
      for (int k = j + 1; k < w; ++k) R[k * LDR + tid] -= x * D[j * LDD + k];
    }
#pragma unroll 16
    for (int k = 0; k < NB; ++k)
      if (k < w) a[(int64_t)(k0 + k) * ld + r] = R[k * LDR + tid];
  }
}

// ---------------------------------------------------------------------------
// SIMT tile update C[rows, cols] -= sum_k A[rows,k] B[cols,k], one task per CTA
// (body in tile_update.cuh).
template <typename T, int TM, int TN, int KT>
__global__ void __launch_bounds__(256) k_update(T* __restrict__ arena,
                                                const T* __restrict__ abuf,
                                                const UpdTask* __restrict__ tasks) {
  __shared__ __align__(16) T As[2][KT][TM];
  __shared__ __align__(16) T Bs[2][KT][TN];
  const UpdTask t = tasks[blockIdx.x];
  tile_update_body<T, TM, TN, KT>(arena + t.c_off, t.ldc, abuf + t.a_off, t.lda,
                                  arena + t.b_off, t.ldb, t.row0, t.col0, t.rowEnd, t.colEnd,
                                  t.k0, t.k1, As, Bs);
}

}  // namespace

// ---------------------------------------------------------------------------

template <typename T>
void launch_zero_lower(T* arena, const ZeroTask* t, int ntask, cudaStream_t s) {
  if (ntask <= 0) return;
  k_zero_lower<T><<<ntask, 256, 0, s>>>(arena, t);
}

template <typename T>
void launch_assemble(T* arena, const double* val, const AsmTask* t, int ntask, const int* acp,
                     const int* arow, const int64_t* asrc, const int* gptr, const EaItem* items,
                     const ChildDesc* cd, const int* maps, cudaStream_t s) {
  if (ntask <= 0) return;
  k_assemble<T><<<ntask, 256, 0, s>>>(arena, val, t, acp, arow, asrc, gptr, items, cd, maps);
}

template <typename T>
void launch_zero_spans(T* arena, const ZeroSpan* t, int ntask, cudaStream_t s) {
  if (ntask <= 0) return;
  k_zero_spans<T><<<ntask, 256, 0, s>>>(arena, t);
}

template <typename T>
void launch_copy_spans(T* dst, const T* src, const CopySpan* t, int ntask, cudaStream_t s) {
  if (ntask <= 0) return;
  k_copy_spans<T><<<ntask, 256, 0, s>>>(dst, src, t);
}

template <typename T>
void launch_init_a(T* arena, const double* val, const int64_t* src, const int64_t* dst,
                   int64_t count, bool atomic, cudaStream_t s) {
  if (count <= 0) return;
  int64_t blocks = std::min<int64_t>((count + 255) / 256, 152 * 32);
  k_init_a<T><<<(int)blocks, 256, 0, s>>>(arena, val, src, dst, count, atomic);
}

template <typename T>
void launch_extend_add(T* arena, const ChildDesc* cd, const EaItem* items, const int* maps,
                       int nitems, cudaStream_t s, bool atomic) {
  if (nitems <= 0) return;
  int blocks = (nitems + 7) / 8;
  k_extend_add<T><<<blocks, 256, 0, s>>>(arena, cd, items, maps, nitems, atomic);
}

template <typename T>
void launch_extend_add_grouped(T* arena, const ChildDesc* cd, const EaItem* items,
                               const int* grp, const int* maps, int ngroups, cudaStream_t s) {
  if (ngroups <= 0) return;
  int blocks = (ngroups + 7) / 8;
  k_extend_add_grouped<T><<<blocks, 256, 0, s>>>(arena, cd, items, grp, maps, ngroups);
}

template <typename T>
static size_t panel_smem() {
  constexpr int NB = Tiles<T>::NB, RT = Tiles<T>::RT;
  return sizeof(T) * ((size_t)NB * (NB + 1) + (size_t)NB * (RT + 1));
}

// Opt-in shared memory sizes; called once per device before any launch (and
// before stream capture).
template <typename T>
void prepare_factor_kernels() {
  constexpr int SM = Tiles<T>::SMALL_M;
  SG_CUDA(cudaFuncSetAttribute(k_small_chol<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)(sizeof(T) * SM * (SM + 1))));
  SG_CUDA(cudaFuncSetAttribute(k_panel_trsm<T, Tiles<T>::NB, Tiles<T>::RT>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)panel_smem<T>()));
}

template <typename T>
void launch_small_chol(T* arena, const SmallTask* t, int ntask, int maxm, unsigned* status,
                       cudaStream_t s) {
  if (ntask <= 0) return;
  size_t smem = sizeof(T) * (size_t)maxm * (maxm + 1);
  k_small_chol<T><<<ntask, 256, smem, s>>>(arena, t, status);
}

template <typename T>
void launch_diag_chol(T* arena, const PanelTask* t, int ntask, unsigned* status,
                      cudaStream_t s) {
  if (ntask <= 0) return;
  k_diag_chol<T, Tiles<T>::NB><<<ntask, 128, 0, s>>>(arena, t, status);
}

template <typename T>
void launch_panel_trsm(T* arena, const PanelTask* t, int ntask, cudaStream_t s) {
  if (ntask <= 0) return;
  constexpr int NB = Tiles<T>::NB, RT = Tiles<T>::RT;
  k_panel_trsm<T, NB, RT><<<ntask, RT, panel_smem<T>(), s>>>(arena, t);
}

template <typename T>
void launch_update(T* arena, const T* abuf, const UpdTask* t, int ntask, cudaStream_t s) {
  if (ntask <= 0) return;
  k_update<T, Tiles<T>::TM, Tiles<T>::TN, 16><<<ntask, 256, 0, s>>>(arena, abuf, t);
}

#define SG_INST(T)                                                                          \
  template void prepare_factor_kernels<T>();                                                 \
  template void launch_zero_lower<T>(T*, const ZeroTask*, int, cudaStream_t);                \
  template void launch_zero_spans<T>(T*, const ZeroSpan*, int, cudaStream_t);                \
  template void launch_copy_spans<T>(T*, const T*, const CopySpan*, int, cudaStream_t);       \
  template void launch_init_a<T>(T*, const double*, const int64_t*, const int64_t*, int64_t, \
                                 bool, cudaStream_t);                                       \
  template void launch_extend_add<T>(T*, const ChildDesc*, const EaItem*, const int*, int,   \
                                     cudaStream_t, bool);                                   \
  template void launch_extend_add_grouped<T>(T*, const ChildDesc*, const EaItem*, const int*, \
                                             const int*, int, cudaStream_t);                \
  template void launch_assemble<T>(T*, const double*, const AsmTask*, int, const int*,       \
                                   const int*, const int64_t*, const int*, const EaItem*,   \
                                   const ChildDesc*, const int*, cudaStream_t);             \
  template void launch_small_chol<T>(T*, const SmallTask*, int, int, unsigned*, cudaStream_t); \
  template void launch_diag_chol<T>(T*, const PanelTask*, int, unsigned*, cudaStream_t);     \
  template void launch_panel_trsm<T>(T*, const PanelTask*, int, cudaStream_t);               \
  template void launch_update<T>(T*, const T*, const UpdTask*, int, cudaStream_t);
SG_INST(float)
SG_INST(double)
#undef SG_INST

}  // namespace sylver_gb300
