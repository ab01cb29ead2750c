// Batched binary128 BLAS: thousands of uneven qgemm / qgemv / qdot problems
// in one persistent launch.  No counterpart in the reference (which has one
// synchronous CPU call per problem); each problem has the semantics of the
// corresponding single call (level1.hpp:80, level2.hpp:85, level3.hpp:215
// with the epilogues of level2.hpp:48 / level3.hpp:107).
//
// Plan (host): every problem is cut into work items of roughly equal cost
// (cost = number of products): qgemm into 32 x 32 C tiles, split along k
// when a tile's k-loop is long; qgemv into groups of 8 rows, split along
// the columns for long rows; qdot into chunks.  Items are sorted by
// decreasing cost (longest-processing-time first).  The item granularity is
// chosen by an autotuner that times a calibration batch once per device
// (cached in memory and in a file).
//
// Execute: a counter reset and one persistent kernel with (SM count x
// resident blocks) blocks; each block takes the next item from an atomic
// queue.  Items of a split group write their partial wide accumulators to
// scratch; the block that completes a group (atomic arrival count) merges
// the partials in index order and applies the epilogue, so results do not
// depend on scheduling.  No block ever waits for another, so nothing can
// spin.  Every final rounding is certified (exact.cuh); the outputs that are
// not (sums cancelling below what the wide accumulator's frame holds) are
// recomputed exactly by the block that finalized them (Kulisch accumulator
// in the shared memory of the operand tiles).  Execute allocates nothing
// and issues one memset and one kernel, so it can be recorded in a CUDA
// graph.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "exact.cuh"
#include "kernels.h"
#include "quadblas_gpu.h"
#include "reduce.cuh"

namespace qb {

constexpr int kBThreads = 256;
constexpr int kBTileMax = 32; // gemm tile edges: 16 (one output per thread) or 32 (2 x 2)
constexpr int kBTK = 16;      // gemm k slice staged in shared memory
constexpr int kBRows = 32;    // gemv rows per item (8 lanes each, 4 per warp)
constexpr int kBRowLanes = 8;

enum : int32_t { kOpGemm = 0, kOpGemv = 1, kOpDot = 2 };

struct BProb {
  int32_t op;
  int32_t nparts;  // items that reduce into each output group (1 = no split)
  int64_t m, n, k;
  q128 alpha, beta;
  const q128* A;
  int64_t sai, sal;  // gemm op(A)(i,l); gemv op(A)(i,j); dot: x stride in sal
  const q128* B;
  int64_t sbl, sbj;  // gemm op(B)(l,j); gemv: x stride in sbl; dot: y stride in sbl
  q128* C;
  int64_t sci, scj;  // gemm C(i,j); gemv: y stride in sci; dot: result
  int64_t part_base;   // first partial-accumulator slot of this problem
  int64_t group_base;  // first arrival counter of this problem
};

struct BItem {
  int32_t prob;
  int32_t part;   // index within the split group
  int64_t i0, j0; // gemm tile origin / gemv first row / unused
  int64_t l0, l1; // k range (gemm), column range (gemv), element range (dot)
  int64_t group;  // output group within the problem (tile / row block / 0)
};

// ---------------------------------------------------------------------------
// device
// ---------------------------------------------------------------------------
template <int T>
struct BTile {
  uint32_t m0[kBTK][T], m1[kBTK][T], m2[kBTK][T], m3[kBTK][T];
  int32_t e[kBTK][T];
  uint32_t sc[kBTK][T];
};

template <int T>
struct BShared {
  static constexpr int kTile = T;
  union {
    struct {
      BTile<T> a, b;
    } t;
    KulischBlock K;  // exact recomputation after an item's accumulation
  } u;
  wacc red[kBThreads / 32];
  int item;
  int last;
  int nlist;
  short list[kBTileMax * kBTileMax];  // uncertified outputs of the current item
};

template <int T>
__device__ __forceinline__ void btile_put(BTile<T>& t, int kk, int idx, q128 v) {
  qop o = qop_unpack(v);
  t.m0[kk][idx] = o.m0;
  t.m1[kk][idx] = o.m1;
  t.m2[kk][idx] = o.m2;
  t.m3[kk][idx] = o.m3;
  t.e[kk][idx] = o.e;
  t.sc[kk][idx] = o.s | (o.cls << 1);
}

template <int T>
__device__ __forceinline__ qop btile_get(const BTile<T>& t, int kk, int idx) {
  qop o;
  o.m0 = t.m0[kk][idx];
  o.m1 = t.m1[kk][idx];
  o.m2 = t.m2[kk][idx];
  o.m3 = t.m3[kk][idx];
  o.e = t.e[kk][idx];
  uint32_t sc = t.sc[kk][idx];
  o.s = sc & 1u;
  o.cls = sc >> 1;
  return o;
}

__device__ __forceinline__ wacc wacc_ldcg(const wacc* p) {
  const uint32_t* q = reinterpret_cast<const uint32_t*>(p);
  wacc a;
  a.w0 = __ldcg(q + 0);
  a.w1 = __ldcg(q + 1);
  a.w2 = __ldcg(q + 2);
  a.w3 = __ldcg(q + 3);
  a.w4 = __ldcg(q + 4);
  a.w5 = __ldcg(q + 5);
  a.w6 = __ldcg(q + 6);
  a.w7 = __ldcg(q + 7);
  a.e = (int32_t)__ldcg(q + 8);
  a.flags = __ldcg(q + 9);
  return a;
}

// Marks one item of a split group done; true in every thread of the block
// that completed the group.  Partials written before the call are visible
// to that block afterwards.
template <class SH>
__device__ __forceinline__ bool group_arrive(SH& sh, int* counter, int nparts) {
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    int prev = atomicAdd(counter, 1);
    sh.last = prev == nparts - 1;
    if (sh.last) *counter = 0;  // ready for the next execution
  }
  __syncthreads();
  bool last = sh.last != 0;
  if (last) __threadfence();
  return last;
}

// A T x T tile of C (T = 16 or 32): thread (tx, ty) of the 16 x 16 grid
// owns the R x R outputs (R*ty + a, R*tx + b), R = T / 16.
template <int T>
__device__ void run_gemm_item(BShared<T>& sh, const BProb& P, const BItem& it, wacc* partials,
                              int* counters) {
  constexpr int R = T / 16;
  constexpr int kUnroll = T == 16 ? 4 : 2;  // k steps in flight (measured: 16-wide 2 % faster at 4)
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const q128 zero = q_zero(0);
  wacc c[R * R];
#pragma unroll
  for (int q = 0; q < R * R; ++q) wacc_init(c[q]);
  for (int64_t l0 = it.l0; l0 < it.l1; l0 += kBTK) {
#pragma unroll
    for (int r = 0; r < R; ++r) {
      int e = tid + r * kBThreads;
      int ar = e >> 4, ak = e & 15;
      int64_t gi = it.i0 + ar, gl = l0 + ak;
      q128 av = (gi < P.m && gl < it.l1) ? ld_cached(P.A + gi * P.sai + gl * P.sal) : zero;
      int bk = e / T, bc = e % T;
      int64_t bl = l0 + bk, gj = it.j0 + bc;
      q128 bv = (bl < it.l1 && gj < P.n) ? ld_cached(P.B + bl * P.sbl + gj * P.sbj) : zero;
      btile_put(sh.u.t.a, ak, ar, av);
      btile_put(sh.u.t.b, bk, bc, bv);
    }
    __syncthreads();
#pragma unroll kUnroll
    for (int kk = 0; kk < kBTK; ++kk) {
      qop a[R], b[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        a[r] = btile_get(sh.u.t.a, kk, R * ty + r);
        b[r] = btile_get(sh.u.t.b, kk, R * tx + r);
      }
#pragma unroll
      for (int q = 0; q < R * R; ++q) wacc_add_product(c[q], a[q / R], b[q % R]);
    }
    __syncthreads();
  }
  if (P.nparts > 1) {
    // partial slot layout: [group][part][thread][R * R]
    wacc* mine = partials + P.part_base + ((it.group * P.nparts + it.part) * kBThreads + tid) * (R * R);
#pragma unroll
    for (int q = 0; q < R * R; ++q) mine[q] = c[q];
    if (!group_arrive(sh, counters + P.group_base + it.group, P.nparts)) return;
#pragma unroll
    for (int q = 0; q < R * R; ++q) wacc_init(c[q]);
    for (int p = 0; p < P.nparts; ++p) {
      const wacc* src = partials + P.part_base + ((it.group * P.nparts + p) * kBThreads + tid) * (R * R);
#pragma unroll
      for (int q = 0; q < R * R; ++q) wacc_merge(c[q], wacc_ldcg(src + q));
    }
  }
  const uint64_t err = 2 * (uint64_t)P.k + 3 * (uint64_t)P.nparts + 2;
#pragma unroll
  for (int q = 0; q < R * R; ++q) {
    const int li = R * ty + q / R, lj = R * tx + q % R;
    int64_t i = it.i0 + li, j = it.j0 + lj;
    if (i < P.m && j < P.n) {
      q128* p = P.C + i * P.sci + j * P.scj;
      q128 r;
      if (wacc_round_certified(c[q], err, r))
        *p = q_epilogue(P.alpha, r, P.beta, *p);
      else
        sh.list[atomicAdd(&sh.nlist, 1)] = (short)(li * T + lj);
    }
  }
  __syncthreads();
  const int cnt = sh.nlist;
  for (int t = 0; t < cnt; ++t) {
    const int64_t i = it.i0 + sh.list[t] / T, j = it.j0 + sh.list[t] % T;
    q128 r = block_exact_dot(sh.u.K, P.k, P.A + i * P.sai, P.sal, P.B + j * P.sbj, P.sbl);
    if (threadIdx.x == 0) {
      q128* p = P.C + i * P.sci + j * P.scj;
      *p = q_epilogue(P.alpha, r, P.beta, *p);
    }
  }
}

// Rows of a qgemv item: 8 lanes per row (4 rows per warp), each lane taking
// every 8th column with four loads in flight; the 8 lanes' accumulators
// merge in three shuffles and the row's first lane finishes it.  (Short rows
// keep most lanes busy: one warp per row spent about as long in its
// 32-lane reduction and one-lane finish as in the products of a row of a
// few hundred columns.)
template <class SH>
__device__ void run_gemv_item(SH& sh, const BProb& P, const BItem& it, wacc* partials,
                              int* counters) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int sl = lane & (kBRowLanes - 1);
  const int r_in = warp * (32 / kBRowLanes) + lane / kBRowLanes;  // row within the item
  const int64_t row = it.i0 + r_in;
  wacc acc;
  wacc_init(acc);
  if (row < P.m) {
    // four loads in flight per lane (A read once, x shared by the rows)
    const q128* Ar = P.A + row * P.sai;
    int64_t j = it.l0 + sl;
    for (; j + 3 * kBRowLanes < it.l1; j += 4 * kBRowLanes) {
      q128 a0 = ld_stream(Ar + j * P.sal), a1 = ld_stream(Ar + (j + kBRowLanes) * P.sal);
      q128 a2 = ld_stream(Ar + (j + 2 * kBRowLanes) * P.sal), a3 = ld_stream(Ar + (j + 3 * kBRowLanes) * P.sal);
      q128 x0 = ld_cached(P.B + j * P.sbl), x1 = ld_cached(P.B + (j + kBRowLanes) * P.sbl);
      q128 x2 = ld_cached(P.B + (j + 2 * kBRowLanes) * P.sbl), x3 = ld_cached(P.B + (j + 3 * kBRowLanes) * P.sbl);
      wacc_add_product(acc, qop_unpack(a0), qop_unpack(x0));
      wacc_add_product(acc, qop_unpack(a1), qop_unpack(x1));
      wacc_add_product(acc, qop_unpack(a2), qop_unpack(x2));
      wacc_add_product(acc, qop_unpack(a3), qop_unpack(x3));
    }
    for (; j < it.l1; j += kBRowLanes)
      wacc_add_product(acc, qop_unpack(ld_stream(Ar + j * P.sal)), qop_unpack(ld_cached(P.B + j * P.sbl)));
  }
  // the 8 lanes of a row into its first lane (lanes of other rows read by a
  // shuffle are not used)
#pragma unroll
  for (int d = kBRowLanes / 2; d >= 1; d >>= 1) {
    wacc b = wacc_shfl_down(acc, d);
    wacc_merge(acc, b);
  }
  const bool lead = sl == 0;
  if (P.nparts > 1) {
    wacc* slot = partials + P.part_base + (it.group * P.nparts + it.part) * kBRows + r_in;
    if (lead) *slot = acc;
    if (!group_arrive(sh, counters + P.group_base + it.group, P.nparts)) return;
    if (lead) {
      wacc_init(acc);
      for (int p = 0; p < P.nparts; ++p)
        wacc_merge(acc, wacc_ldcg(partials + P.part_base + (it.group * P.nparts + p) * kBRows + r_in));
    }
  }
  if (lead && row < P.m) {
    q128* yp = P.C + row * P.sci;
    q128 r;
    if (wacc_round_certified(acc, 2 * (uint64_t)P.n + 3 * (33 * (uint64_t)P.nparts + 2), r))
      *yp = q_epilogue(P.alpha, r, P.beta, *yp);
    else
      sh.list[atomicAdd(&sh.nlist, 1)] = (short)r_in;
  }
  __syncthreads();
  const int cnt = sh.nlist;
  for (int t = 0; t < cnt; ++t) {
    const int64_t i = it.i0 + sh.list[t];
    q128 r = block_exact_dot(sh.u.K, P.n, P.A + i * P.sai, P.sal, P.B, P.sbl);
    if (threadIdx.x == 0) {
      q128* yp = P.C + i * P.sci;
      *yp = q_epilogue(P.alpha, r, P.beta, *yp);
    }
  }
}

template <class SH>
__device__ void run_dot_item(SH& sh, const BProb& P, const BItem& it, wacc* partials,
                             int* counters) {
  wacc acc;
  wacc_init(acc);
  int64_t i = it.l0 + threadIdx.x;
  for (; i + 3 * kBThreads < it.l1; i += 4 * kBThreads) {
    q128 x0 = ld_stream(P.A + i * P.sal), x1 = ld_stream(P.A + (i + kBThreads) * P.sal);
    q128 x2 = ld_stream(P.A + (i + 2 * kBThreads) * P.sal), x3 = ld_stream(P.A + (i + 3 * kBThreads) * P.sal);
    q128 y0 = ld_stream(P.B + i * P.sbl), y1 = ld_stream(P.B + (i + kBThreads) * P.sbl);
    q128 y2 = ld_stream(P.B + (i + 2 * kBThreads) * P.sbl), y3 = ld_stream(P.B + (i + 3 * kBThreads) * P.sbl);
    wacc_add_product(acc, qop_unpack(x0), qop_unpack(y0));
    wacc_add_product(acc, qop_unpack(x1), qop_unpack(y1));
    wacc_add_product(acc, qop_unpack(x2), qop_unpack(y2));
    wacc_add_product(acc, qop_unpack(x3), qop_unpack(y3));
  }
  for (; i < it.l1; i += kBThreads)
    wacc_add_product(acc, qop_unpack(ld_cached(P.A + i * P.sal)), qop_unpack(ld_cached(P.B + i * P.sbl)));
  wacc_block_reduce(acc, sh.red);
  if (P.nparts > 1) {
    if (threadIdx.x == 0) partials[P.part_base + it.part] = acc;
    if (!group_arrive(sh, counters + P.group_base, P.nparts)) return;
    if (threadIdx.x == 0) {
      wacc_init(acc);
      for (int p = 0; p < P.nparts; ++p) wacc_merge(acc, wacc_ldcg(partials + P.part_base + p));
    }
  }
  if (threadIdx.x == 0) {
    q128 r;
    const bool ok = wacc_round_certified(acc, 2 * (uint64_t)P.n + 3 * (257 * (uint64_t)P.nparts + 2), r);
    if (ok) *P.C = r;
    sh.nlist = ok ? 0 : 1;
  }
  __syncthreads();
  if (sh.nlist) {
    q128 r = block_exact_dot(sh.u.K, P.n, P.A, P.sal, P.B, P.sbl);
    if (threadIdx.x == 0) *P.C = r;
  }
}

// Resident blocks per SM: four for the 16-wide tile (at most 64 registers; the
// streaming qgemv and qdot items gain most from the extra loads in flight),
// two for the 32-wide tile, whose four wide accumulators per thread need more.
template <int T>
__global__ void __launch_bounds__(kBThreads, T == 16 ? 4 : 2)
    batched_persistent_kernel(const BProb* __restrict__ probs, const BItem* __restrict__ items,
                              int64_t nitems, int* queue, int* counters, wacc* partials) {
  __shared__ BShared<T> sh;
  while (true) {
    if (threadIdx.x == 0) {
      sh.item = atomicAdd(queue, 1);
      sh.nlist = 0;
    }
    __syncthreads();
    const int64_t idx = sh.item;
    __syncthreads();
    if (idx >= nitems) break;
    const BItem it = items[idx];
    const BProb P = probs[it.prob];
    if (P.op == kOpGemm)
      run_gemm_item(sh, P, it, partials, counters);
    else if (P.op == kOpGemv)
      run_gemv_item(sh, P, it, partials, counters);
    else
      run_dot_item(sh, P, it, partials, counters);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// host: plan, execute, autotune
// ---------------------------------------------------------------------------
struct BatchPlan {
  int device = -1;
  int64_t nitems = 0, nprobs = 0, ngroups = 0, nparts = 0;
  int64_t grain = 0;
  int tile = 32;  // gemm C tile edge (16 or 32)
  BProb* d_probs = nullptr;
  BItem* d_items = nullptr;
  int* d_counters = nullptr;  // [0] = queue head, [1..] group counters
  wacc* d_partials = nullptr;
  int blocks = 0;
  // qgemm problems on the grouped residue path (method 2, large enough)
  int64_t n_ozaki = 0;
  OzakiGroup grp = {};
  void* d_grp = nullptr;  // one allocation: rows, tiles, problems, stacked operands, scratch
};

static bool is_trans(char t) { return t == 'T' || t == 't' || t == 'C' || t == 'c'; }
static bool is_col(char l) { return l == 'C' || l == 'c'; }

static int resolve(const qblas_problem& q, BProb& P) {
  memset(&P, 0, sizeof(P));
  memcpy(&P.alpha, q.alpha, 16);
  memcpy(&P.beta, q.beta, 16);
  P.A = (const q128*)q.A;
  P.B = (const q128*)q.B;
  P.C = (q128*)q.C;
  if (!q.C) return kErrInvalidValue;
  if (q.op == QBLAS_OP_GEMM) {
    if (q.m < 0 || q.n < 0 || q.k < 0) return kErrInvalidValue;
    bool col = is_col(q.layout), ta = is_trans(q.transa), tb = is_trans(q.transb);
    int64_t ar = ta ? q.k : q.m, ac = ta ? q.m : q.k, br = tb ? q.n : q.k, bc = tb ? q.k : q.n;
    if (!col) {
      if (q.lda < std::max<int64_t>(1, ac) || q.ldb < std::max<int64_t>(1, bc) ||
          q.ldc < std::max<int64_t>(1, q.n))
        return kErrInvalidValue;
      P.sai = ta ? 1 : q.lda;
      P.sal = ta ? q.lda : 1;
      P.sbl = tb ? 1 : q.ldb;
      P.sbj = tb ? q.ldb : 1;
      P.sci = q.ldc;
      P.scj = 1;
    } else {
      if (q.lda < std::max<int64_t>(1, ar) || q.ldb < std::max<int64_t>(1, br) ||
          q.ldc < std::max<int64_t>(1, q.m))
        return kErrInvalidValue;
      P.sai = ta ? q.lda : 1;
      P.sal = ta ? 1 : q.lda;
      P.sbl = tb ? q.ldb : 1;
      P.sbj = tb ? 1 : q.ldb;
      P.sci = 1;
      P.scj = q.ldc;
    }
    P.op = kOpGemm;
    P.m = q.m;
    P.n = q.n;
    P.k = q.k;
  } else if (q.op == QBLAS_OP_GEMV) {
    int64_t m = q.m, n = q.n;
    bool col = is_col(q.layout);
    if (m < 0 || n < 0) return kErrInvalidValue;
    if (is_trans(q.transa)) {
      std::swap(m, n);
      col = !col;
    }
    if (!col) {
      if (q.lda < std::max<int64_t>(1, n)) return kErrInvalidValue;
      P.sai = q.lda;
      P.sal = 1;
    } else {
      if (q.lda < std::max<int64_t>(1, m)) return kErrInvalidValue;
      P.sai = 1;
      P.sal = q.lda;
    }
    if ((m > 0 && n > 0) && (q.ldb <= 0 || q.ldc <= 0)) return kErrInvalidValue;
    P.op = kOpGemv;
    P.m = m;
    P.n = n;
    P.sbl = q.ldb;  // incx
    P.sci = q.ldc;  // incy
  } else if (q.op == QBLAS_OP_DOT) {
    if (q.n < 0 || (q.n > 0 && (q.lda <= 0 || q.ldb <= 0))) return kErrInvalidValue;
    P.op = kOpDot;
    P.n = q.n;
    P.sal = q.lda;  // incx
    P.sbl = q.ldb;  // incy
  } else {
    return kErrInvalidValue;
  }
  return kOk;
}

static int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Items of all problems for a granularity `grain` (products per item) and a
// gemm tile edge `tile`.
static int build_items(std::vector<BProb>& probs, int64_t grain, int tile, std::vector<BItem>& items,
                       std::vector<int64_t>& cost, int64_t& ngroups, int64_t& nparts_total) {
  items.clear();
  cost.clear();
  ngroups = 0;
  nparts_total = 0;
  for (size_t pi = 0; pi < probs.size(); ++pi) {
    BProb& P = probs[pi];
    P.group_base = 1 + ngroups;  // counter 0 is the queue head
    P.part_base = nparts_total;
    P.nparts = 1;
    if (P.op == kOpGemm) {
      if (P.m == 0 || P.n == 0 || P.k == 0) continue;  // level3.hpp:221
      int64_t tm = cdiv(P.m, tile), tn = cdiv(P.n, tile);
      int64_t kslices = cdiv(P.k, kBTK);
      int64_t per = (int64_t)tile * tile * P.k;
      int64_t parts = std::min<int64_t>(std::max<int64_t>(1, cdiv(per, grain)), kslices);
      int64_t kper = cdiv(kslices, parts) * kBTK;
      parts = cdiv(P.k, kper);
      P.nparts = (int32_t)parts;
      for (int64_t a = 0; a < tm; ++a)
        for (int64_t b = 0; b < tn; ++b)
          for (int64_t p = 0; p < parts; ++p) {
            BItem it;
            it.prob = (int32_t)pi;
            it.part = (int32_t)p;
            it.i0 = a * tile;
            it.j0 = b * tile;
            it.l0 = p * kper;
            it.l1 = std::min(P.k, (p + 1) * kper);
            it.group = a * tn + b;
            items.push_back(it);
            cost.push_back((int64_t)tile * tile * (it.l1 - it.l0));
          }
      if (parts > 1) {
        ngroups += tm * tn;
        nparts_total += tm * tn * parts * tile * tile;  // one wide accumulator per output
      }
    } else if (P.op == kOpGemv) {
      if (P.m == 0 || P.n == 0) continue;  // level2.hpp:21,61
      int64_t rb = cdiv(P.m, kBRows);
      int64_t per = (int64_t)kBRows * P.n;
      int64_t parts = std::min<int64_t>(std::max<int64_t>(1, cdiv(per, grain)), cdiv(P.n, 256));
      int64_t cper = cdiv(P.n, parts);
      parts = cdiv(P.n, cper);
      P.nparts = (int32_t)parts;
      for (int64_t a = 0; a < rb; ++a)
        for (int64_t p = 0; p < parts; ++p) {
          BItem it;
          it.prob = (int32_t)pi;
          it.part = (int32_t)p;
          it.i0 = a * kBRows;
          it.j0 = 0;
          it.l0 = p * cper;
          it.l1 = std::min(P.n, (p + 1) * cper);
          it.group = a;
          items.push_back(it);
          cost.push_back((int64_t)kBRows * (it.l1 - it.l0));
        }
      if (parts > 1) {
        ngroups += rb;
        nparts_total += rb * parts * kBRows;
      }
    } else {
      int64_t parts = std::max<int64_t>(1, cdiv(P.n, grain));
      if (P.n == 0) parts = 1;
      int64_t cper = std::max<int64_t>(1, cdiv(P.n, parts));
      parts = P.n == 0 ? 1 : cdiv(P.n, cper);
      P.nparts = (int32_t)parts;
      for (int64_t p = 0; p < parts; ++p) {
        BItem it;
        it.prob = (int32_t)pi;
        it.part = (int32_t)p;
        it.i0 = it.j0 = 0;
        it.l0 = p * cper;
        it.l1 = std::min(P.n, (p + 1) * cper);
        it.group = 0;
        items.push_back(it);
        cost.push_back(2 * (it.l1 - it.l0) + 256);
      }
      if (parts > 1) {
        ngroups += 1;
        nparts_total += parts;
      }
    }
  }
  // longest processing time first (stable, so equal costs keep problem order)
  std::vector<int64_t> order(items.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = (int64_t)i;
  std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return cost[a] > cost[b]; });
  std::vector<BItem> sorted(items.size());
  for (size_t i = 0; i < order.size(); ++i) sorted[i] = items[order[i]];
  items.swap(sorted);
  return kOk;
}

static int cuda_rc(cudaError_t e) {
  if (e == cudaSuccess) return kOk;
  cudaGetLastError();
  if (e == cudaErrorMemoryAllocation) return kErrNoMemory;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return kErrNoDevice;
  return kErrCuda;
}

static int plan_free(BatchPlan* p) {
  if (!p) return kOk;
  cudaFree(p->d_probs);
  cudaFree(p->d_items);
  cudaFree(p->d_counters);
  cudaFree(p->d_partials);
  cudaFree(p->d_grp);
  delete p;
  return kOk;
}

// ---- qgemm problems on the grouped residue path ----------------------------
// Under method 2 a qgemm problem with m n k at or above the threshold runs on
// the tensor cores, like its single call: all such problems of the batch go
// through one chain of launches (launch_gemm_ozaki_grouped) after the
// persistent kernel, in the same stream, so the plan stays one graph.  The
// digits are those of the single call; the moduli are taken for the largest
// k of the group (more moduli than a problem needs reconstruct the same
// integer), so every output is bit-identical to its single call's.
constexpr int64_t kRouteMaxK = 8192;  // one k pass

static std::atomic<int64_t> g_route_min{0};  // quadblas_batch_set_ozaki_min; 0: environment or default

static int64_t route_min_products() {
  const int64_t set = g_route_min.load();
  if (set > 0) return set;
  static const int64_t v = [] {
    const char* e = getenv("QBLAS_BATCH_OZAKI_MIN");
    const long long x = e ? atoll(e) : 0;
    return x > 0 ? (int64_t)x : (int64_t)1 << 20;
  }();
  return v;
}

static int64_t rup64(int64_t v, int64_t a) { return (v + a - 1) / a * a; }

static bool routed(const BProb& P) {
  return P.op == kOpGemm && P.m > 0 && P.n > 0 && P.k > 0 && batch_gemm_routed(P.m, P.n, P.k);
}

// The stacked rows, tiles and problem table of the routed problems, the
// stacked operand buffers (zeroed) and the scratch, in one allocation.
static int build_group(const std::vector<BProb>& probs, const std::vector<char>& route, BatchPlan* p) {
  std::vector<OzakiGroupRow> rows_a, rows_b;
  std::vector<OzakiGroupTile> tiles;
  std::vector<OzakiGroupProb> gp;
  int64_t kmax = 0;
  for (size_t i = 0; i < probs.size(); ++i)
    if (route[i]) kmax = std::max(kmax, probs[i].k);
  if (kmax == 0) return kOk;
  const int64_t k_pad = rup64(kmax, 64);
  for (size_t i = 0; i < probs.size(); ++i) {
    if (!route[i]) continue;
    const BProb& P = probs[i];
    const int64_t m_pad = rup64(P.m, 128), n_pad = rup64(P.n, 256);
    const int32_t a0 = (int32_t)(rows_a.size() / 128), b0 = (int32_t)(rows_b.size() / 256);
    for (int64_t r = 0; r < m_pad; ++r)
      rows_a.push_back(r < P.m ? OzakiGroupRow{P.A + r * P.sai, P.sal, P.k} : OzakiGroupRow{nullptr, 0, 0});
    for (int64_t c = 0; c < n_pad; ++c)
      rows_b.push_back(c < P.n ? OzakiGroupRow{P.B + c * P.sbj, P.sbl, P.k} : OzakiGroupRow{nullptr, 0, 0});
    const int32_t pi = (int32_t)gp.size();
    for (int64_t a = 0; a < m_pad / 128; ++a)
      for (int64_t b = 0; b < n_pad / 256; ++b)
        tiles.push_back(OzakiGroupTile{a0 + (int32_t)a, b0 + (int32_t)b, pi, (int32_t)(128 * a), (int32_t)(256 * b), {0, 0, 0}});
    OzakiGroupProb q;
    q.C = P.C;
    q.sci = P.sci;
    q.scj = P.scj;
    q.m = P.m;
    q.n = P.n;
    q.k = P.k;
    q.alpha = P.alpha;
    q.beta = P.beta;
    q.A = P.A;
    q.sai = P.sai;
    q.sal = P.sal;
    q.B = P.B;
    q.sbl = P.sbl;
    q.sbj = P.sbj;
    gp.push_back(q);
  }
  OzakiGroup& G = p->grp;
  G.rows_a = (int64_t)rows_a.size();
  G.rows_b = (int64_t)rows_b.size();
  G.k_pad = k_pad;
  G.ntiles = (int64_t)tiles.size();
  G.k_max = kmax;
  G.digits = gemm_digits_setting(kRouteMaxK);
  G.bits = gemm_bits_setting();
  const size_t sb = ozaki_group_scratch_bytes(G.rows_a, G.rows_b, k_pad, G.ntiles, kmax, G.digits, G.bits);
  if (sb == 0) return kErrInvalidValue;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t o_rows = 0, o_tiles = o_rows + al(sizeof(OzakiGroupRow) * (rows_a.size() + rows_b.size()));
  const size_t o_probs = o_tiles + al(sizeof(OzakiGroupTile) * tiles.size());
  const size_t o_a = o_probs + al(sizeof(OzakiGroupProb) * gp.size());
  const size_t o_b = o_a + al((size_t)G.rows_a * k_pad * 16);
  const size_t o_s = o_b + al((size_t)G.rows_b * k_pad * 16);
  const size_t total = o_s + sb;
  int rc = cuda_rc(dev_malloc(&p->d_grp, total));
  if (rc) return rc;
  char* b = static_cast<char*>(p->d_grp);
  std::vector<OzakiGroupRow> all(rows_a);
  all.insert(all.end(), rows_b.begin(), rows_b.end());
  if ((rc = cuda_rc(cudaMemcpy(b + o_rows, all.data(), sizeof(OzakiGroupRow) * all.size(), cudaMemcpyHostToDevice))) ||
      (rc = cuda_rc(cudaMemcpy(b + o_tiles, tiles.data(), sizeof(OzakiGroupTile) * tiles.size(),
                               cudaMemcpyHostToDevice))) ||
      (rc = cuda_rc(cudaMemcpy(b + o_probs, gp.data(), sizeof(OzakiGroupProb) * gp.size(), cudaMemcpyHostToDevice))) ||
      (rc = cuda_rc(cudaMemset(b + o_a, 0, o_s - o_a))))
    return rc;
  G.rows = reinterpret_cast<const OzakiGroupRow*>(b + o_rows);
  G.tiles = reinterpret_cast<const OzakiGroupTile*>(b + o_tiles);
  G.probs = reinterpret_cast<const OzakiGroupProb*>(b + o_probs);
  G.a_all = reinterpret_cast<q128*>(b + o_a);
  G.b_all = reinterpret_cast<q128*>(b + o_b);
  G.scratch = b + o_s;
  p->n_ozaki = (int64_t)gp.size();
  return kOk;
}

static const void* persistent_kernel(int tile) {
  return tile == 16 ? (const void*)batched_persistent_kernel<16> : (const void*)batched_persistent_kernel<32>;
}

// route = false (the autotuner's calibration): every problem on the persistent kernel.
static int plan_build(const qblas_problem* problems, int64_t count, int64_t grain, int tile, BatchPlan** out,
                      bool route_ok = true) {
  *out = nullptr;
  if (count < 0 || (count > 0 && !problems) || (tile != 16 && tile != 32)) return kErrInvalidValue;
  std::vector<BProb> probs((size_t)count);
  std::vector<char> route((size_t)count, 0);
  for (int64_t i = 0; i < count; ++i) {
    int rc = resolve(problems[i], probs[i]);
    if (rc) return rc;
    route[i] = route_ok && routed(probs[i]) ? 1 : 0;
  }
  // the persistent kernel's items leave out the routed problems (a problem
  // with m = 0 has no items)
  std::vector<BProb> kept(probs);
  for (int64_t i = 0; i < count; ++i)
    if (route[i]) kept[i].m = 0;
  std::vector<BItem> items;
  std::vector<int64_t> cost;
  int64_t ngroups = 0, nparts = 0;
  build_items(kept, grain, tile, items, cost, ngroups, nparts);
  BatchPlan* p = new BatchPlan();
  cudaGetDevice(&p->device);
  p->nitems = (int64_t)items.size();
  p->nprobs = count;
  p->ngroups = ngroups;
  p->nparts = nparts;
  p->grain = grain;
  p->tile = tile;
  int rc = kOk;
  if ((rc = cuda_rc(dev_malloc((void**)&p->d_probs, sizeof(BProb) * std::max<int64_t>(1, count)))) ||
      (rc = cuda_rc(dev_malloc((void**)&p->d_items, sizeof(BItem) * std::max<int64_t>(1, p->nitems)))) ||
      (rc = cuda_rc(dev_malloc((void**)&p->d_counters, sizeof(int) * (1 + ngroups)))) ||
      (rc = cuda_rc(dev_malloc((void**)&p->d_partials, sizeof(wacc) * std::max<int64_t>(1, nparts))))) {
    plan_free(p);
    return rc;
  }
  if ((rc = build_group(probs, route, p))) {
    plan_free(p);
    return rc;
  }
  if (count > 0 &&
      (rc = cuda_rc(cudaMemcpy(p->d_probs, kept.data(), sizeof(BProb) * count, cudaMemcpyHostToDevice)))) {
    plan_free(p);
    return rc;
  }
  if (p->nitems > 0 && (rc = cuda_rc(cudaMemcpy(p->d_items, items.data(), sizeof(BItem) * p->nitems,
                                                 cudaMemcpyHostToDevice)))) {
    plan_free(p);
    return rc;
  }
  if ((rc = cuda_rc(cudaMemset(p->d_counters, 0, sizeof(int) * (1 + ngroups))))) {
    plan_free(p);
    return rc;
  }
  int per_sm = resident_blocks_per_sm(persistent_kernel(tile), kBThreads, 0);
  p->blocks = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)device_sm_count() * per_sm, p->nitems));
  *out = p;
  return kOk;
}

static int plan_execute(BatchPlan* p, cudaStream_t s) {
  if (!p) return kErrInvalidValue;
  if (p->n_ozaki > 0) {
    const int rc = cuda_rc(launch_gemm_ozaki_grouped(p->grp, s));
    if (rc) return rc;
  }
  if (p->nitems == 0) return kOk;
  cudaError_t e = cudaMemsetAsync(p->d_counters, 0, sizeof(int) * (1 + p->ngroups), s);
  if (e != cudaSuccess) return cuda_rc(e);
  if (p->tile == 16)
    batched_persistent_kernel<16><<<p->blocks, kBThreads, 0, s>>>(p->d_probs, p->d_items, p->nitems, p->d_counters,
                                                                  p->d_counters, p->d_partials);
  else
    batched_persistent_kernel<32><<<p->blocks, kBThreads, 0, s>>>(p->d_probs, p->d_items, p->nitems, p->d_counters,
                                                                  p->d_counters, p->d_partials);
  return cuda_rc(cudaGetLastError());
}

// ---- autotuner ------------------------------------------------------------
// Candidates: gemm tile edge (16, 32) x granularity (products per work item,
// 2^14 .. 2^20).  The tuner times a fixed calibration batch (the shapes of
// the batched benchmark, fewer problems, data generated on the device) at
// each pair and keeps the fastest.  The result is cached per device in
// memory and in the file $QBLAS_AUTOTUNE_CACHE (default
// $HOME/.cache/qblas_gb300_autotune.txt) as "<device name> <grain> <tile>".
static const int64_t kGrains[] = {1 << 14, 1 << 15, 1 << 16, 1 << 17, 1 << 18, 1 << 19, 1 << 20};
static const int kTiles[] = {16, 32};
static const int64_t kDefaultGrain = 1 << 16;
static const int kDefaultTile = 32;
static std::mutex g_tune_mu;
struct TuneSetting {
  int64_t grain;
  int tile;
};
static TuneSetting g_setting[64] = {};

static std::string cache_path() {
  const char* e = getenv("QBLAS_AUTOTUNE_CACHE");
  if (e && *e) return e;
  const char* h = getenv("HOME");
  return std::string(h ? h : "/tmp") + "/.cache/qblas_gb300_autotune.txt";
}

static std::string device_key(int dev) {
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return "unknown";
  std::string k = prop.name;
  for (char& c : k)
    if (c == ' ') c = '_';
  return k + "_sm" + std::to_string(prop.multiProcessorCount);
}

// The device's setting: tuned or set in this process, else the last line of
// the cache file for this device, else the defaults.  A line without a tile
// (an older cache) keeps the default tile.
static TuneSetting cached_setting(int dev) {
  std::lock_guard<std::mutex> l(g_tune_mu);
  if (dev < 0 || dev >= 64) return {kDefaultGrain, kDefaultTile};
  if (g_setting[dev].grain) return g_setting[dev];
  FILE* f = fopen(cache_path().c_str(), "r");
  if (f) {
    char line[512], name[256];
    std::string key = device_key(dev);
    while (fgets(line, sizeof line, f)) {
      long long g = 0;
      int t = kDefaultTile;
      int n = sscanf(line, "%255s %lld %d", name, &g, &t);
      if (n >= 2 && key == name && g >= 256 && (t == 16 || t == 32)) g_setting[dev] = {(int64_t)g, t};
    }
    fclose(f);
  }
  if (!g_setting[dev].grain) return {kDefaultGrain, kDefaultTile};
  return g_setting[dev];
}

__global__ void fill_bits_kernel(uint64_t* p, int64_t n, uint64_t seed) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  // splitmix64 bits; element i is a binary128 with a random significand and
  // an exponent near 1 (|x| in [1, 2)), sign from the hash
  uint64_t z = seed + (uint64_t)i * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  if (i & 1)
    p[i] = (z & 0x8000FFFFFFFFFFFFull) | (0x3FFFull << 48);
  else
    p[i] = z;
}

static int run_autotune(int dev, TuneSetting* best_out) {
  // calibration batch: 800 each of gemm (m, n, k in 8..256), gemv (m, n in
  // 16..2048) and dot (n in 64..65536), log-uniform sizes (about 2.5 GB)
  const int nper = 800;
  uint64_t st = 0x2545F4914F6CDD1Dull;
  auto rnd = [&]() {
    st ^= st << 13;
    st ^= st >> 7;
    st ^= st << 17;
    return st;
  };
  auto logu = [&](double lo, double hi) {
    double u = (double)(rnd() >> 11) * (1.0 / 9007199254740992.0);
    double v = exp(log(lo) + u * (log(hi + 1) - log(lo)));
    int64_t r = (int64_t)v;
    return std::min<int64_t>(std::max<int64_t>(r, (int64_t)lo), (int64_t)hi);
  };
  std::vector<qblas_problem> probs;
  int64_t total = 0;
  struct Sz {
    int op;
    int64_t m, n, k;
  };
  std::vector<Sz> sz;
  for (int i = 0; i < nper; ++i) {
    Sz a{QBLAS_OP_GEMM, logu(8, 256), logu(8, 256), logu(8, 256)};
    Sz b{QBLAS_OP_GEMV, logu(16, 2048), logu(16, 2048), 0};
    Sz c{QBLAS_OP_DOT, 0, logu(64, 65536), 0};
    sz.push_back(a);
    sz.push_back(b);
    sz.push_back(c);
  }
  for (const Sz& z : sz) {
    if (z.op == QBLAS_OP_GEMM) total += z.m * z.k + z.k * z.n + z.m * z.n;
    if (z.op == QBLAS_OP_GEMV) total += z.m * z.n + z.n + z.m;
    if (z.op == QBLAS_OP_DOT) total += 2 * z.n + 1;
  }
  uint64_t* buf = nullptr;
  if (dev_malloc((void**)&buf, (size_t)total * 16) != cudaSuccess) {
    cudaGetLastError();
    return kErrNoMemory;
  }
  fill_bits_kernel<<<(unsigned)((2 * total + 255) / 256), 256>>>(buf, 2 * total, 12345);
  int64_t off = 0;
  uint64_t one[2] = {0, 0x3FFF000000000000ull}, zero[2] = {0, 0};
  for (const Sz& z : sz) {
    qblas_problem q;
    memset(&q, 0, sizeof(q));
    q.op = z.op;
    q.layout = 'R';
    q.transa = q.transb = 'N';
    memcpy(q.alpha, one, 16);
    memcpy(q.beta, zero, 16);
    q128* b = (q128*)buf + off;
    if (z.op == QBLAS_OP_GEMM) {
      q.m = z.m; q.n = z.n; q.k = z.k;
      q.A = b; q.lda = z.k;
      q.B = b + z.m * z.k; q.ldb = z.n;
      q.C = b + z.m * z.k + z.k * z.n; q.ldc = z.n;
      off += z.m * z.k + z.k * z.n + z.m * z.n;
    } else if (z.op == QBLAS_OP_GEMV) {
      q.m = z.m; q.n = z.n;
      q.A = b; q.lda = z.n;
      q.B = b + z.m * z.n; q.ldb = 1;
      q.C = b + z.m * z.n + z.n; q.ldc = 1;
      off += z.m * z.n + z.n + z.m;
    } else {
      q.n = z.n;
      q.A = b; q.lda = 1;
      q.B = b + z.n; q.ldb = 1;
      q.C = b + 2 * z.n;
      off += 2 * z.n + 1;
    }
    probs.push_back(q);
  }
  cudaStream_t s;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best_ms = 1e30f;
  TuneSetting best = {kDefaultGrain, kDefaultTile};
  for (int t : kTiles)
    for (int64_t g : kGrains) {
      BatchPlan* p = nullptr;
      if (plan_build(probs.data(), (int64_t)probs.size(), g, t, &p, false) != kOk) continue;
      plan_execute(p, s);  // warm-up
      cudaEventRecord(e0, s);
      for (int r = 0; r < 3; ++r) plan_execute(p, s);
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < best_ms) {
        best_ms = ms;
        best = {g, t};
      }
      plan_free(p);
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  cudaFree(buf);
  *best_out = best;
  {
    std::lock_guard<std::mutex> l(g_tune_mu);
    g_setting[dev] = best;
  }
  std::string path = cache_path();
  std::string dir = path.substr(0, path.find_last_of('/'));
  std::string cmd = "mkdir -p '" + dir + "' 2>/dev/null";
  if (system(cmd.c_str()) == 0) {
    FILE* f = fopen(path.c_str(), "a");
    if (f) {
      fprintf(f, "%s %lld %d\n", device_key(dev).c_str(), (long long)best.grain, best.tile);
      fclose(f);
    }
  }
  return kOk;
}

bool batch_gemm_routed(int64_t m, int64_t n, int64_t k) {
  if (gemm_method_setting() != 2 || ozaki_scheme_setting() == 1 || k > kRouteMaxK) return false;
  if ((double)m * (double)n * (double)k < (double)route_min_products()) return false;
  const int d = gemm_digits_setting(kRouteMaxK), b = gemm_bits_setting();
  return gemm_digits_setting(k) == d && ozaki_uses_crt(kRouteMaxK, d, b, 2);
}

}  // namespace qb

#define QBLAS_EXPORT extern "C" __attribute__((visibility("default")))

QBLAS_EXPORT int quadblas_batch_plan(const qblas_problem* problems, int64_t count, void** plan) {
  if (!plan) return QBLAS_ERR_INVALID_VALUE;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return QBLAS_ERR_NO_DEVICE;
  }
  qb::BatchPlan* p = nullptr;
  const qb::TuneSetting t = qb::cached_setting(dev);
  int rc = qb::plan_build(problems, count, t.grain, t.tile, &p);
  *plan = p;
  return rc;
}

QBLAS_EXPORT int quadblas_batch_execute(void* plan, void* stream) {
  return qb::plan_execute(static_cast<qb::BatchPlan*>(plan), static_cast<cudaStream_t>(stream));
}

// One batch, once: plan, execute on `stream`, wait for the stream, free the plan.
QBLAS_EXPORT int quadblas_qgemm_batched_dev(const qblas_problem* problems, int64_t count, void* stream) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return QBLAS_ERR_NO_DEVICE;
  }
  qb::BatchPlan* p = nullptr;
  const qb::TuneSetting t = qb::cached_setting(dev);
  int rc = qb::plan_build(problems, count, t.grain, t.tile, &p);
  if (rc) return rc;
  rc = qb::plan_execute(p, static_cast<cudaStream_t>(stream));
  const cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
  qb::plan_free(p);
  if (rc) return rc;
  return qb::cuda_rc(e);
}

QBLAS_EXPORT int quadblas_batch_destroy(void* plan) {
  return qb::plan_free(static_cast<qb::BatchPlan*>(plan));
}

QBLAS_EXPORT int quadblas_batch_info(void* plan, int64_t* info4) {
  qb::BatchPlan* p = static_cast<qb::BatchPlan*>(plan);
  if (!p || !info4) return QBLAS_ERR_INVALID_VALUE;
  info4[0] = p->nitems;
  info4[1] = p->grain;
  info4[2] = p->blocks;
  info4[3] = p->ngroups;
  return QBLAS_OK;
}

QBLAS_EXPORT int quadblas_batch_info_ex(void* plan, int64_t* info, int64_t n) {
  qb::BatchPlan* p = static_cast<qb::BatchPlan*>(plan);
  if (!p || (n > 0 && !info) || n < 0) return QBLAS_ERR_INVALID_VALUE;
  const int64_t v[7] = {p->nitems, p->grain, p->blocks, p->ngroups, p->tile, p->n_ozaki, p->grp.ntiles};
  for (int64_t i = 0; i < n && i < 7; ++i) info[i] = v[i];
  return QBLAS_OK;
}

QBLAS_EXPORT int quadblas_batch_autotune(int64_t* grain_out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return QBLAS_ERR_NO_DEVICE;
  }
  qb::TuneSetting t = {0, 0};
  int rc = qb::run_autotune(dev, &t);
  if (grain_out) *grain_out = t.grain;
  return rc;
}

QBLAS_EXPORT int quadblas_batch_setting(int64_t* grain, int* tile) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return QBLAS_ERR_NO_DEVICE;
  }
  const qb::TuneSetting t = qb::cached_setting(dev);
  if (grain) *grain = t.grain;
  if (tile) *tile = t.tile;
  return QBLAS_OK;
}

// Sets the current device's granularity (>= 256 products per item) and gemm
// tile edge (16 or 32; 0 keeps the current edge) for plans built afterwards.
QBLAS_EXPORT int quadblas_batch_configure(int64_t grain, int tile) {
  int dev = 0;
  if (grain < 256 || (tile != 0 && tile != 16 && tile != 32) || cudaGetDevice(&dev) != cudaSuccess || dev < 0 ||
      dev >= 64) {
    cudaGetLastError();
    return QBLAS_ERR_INVALID_VALUE;
  }
  const qb::TuneSetting cur = qb::cached_setting(dev);
  std::lock_guard<std::mutex> l(qb::g_tune_mu);
  qb::g_setting[dev] = {grain, tile ? tile : cur.tile};
  return QBLAS_OK;
}

QBLAS_EXPORT int quadblas_batch_set_grain(int64_t grain) { return quadblas_batch_configure(grain, 0); }

// Smallest m*n*k of a qgemm problem that plans built afterwards give to the
// grouped tensor-core path under the Ozaki method (0: QBLAS_BATCH_OZAKI_MIN or 2^20).
QBLAS_EXPORT int quadblas_batch_set_ozaki_min(int64_t products) {
  if (products < 0) return QBLAS_ERR_INVALID_VALUE;
  qb::g_route_min.store(products);
  return QBLAS_OK;
}
