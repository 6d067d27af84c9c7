// Neighbor search on the GPU.
//
// mkNNIndxCB (reference src/nn.cpp:128-258): the mean-distance-ordered search of
// Ra & Kim (1993).  Locations are sorted by u = x + y; each location walks the
// sorted order alternately down and up from its own position, stops a direction
// once ((x_q + y_q) - x_j - y_j)^2 > 2*worst, and accepts predecessors (original
// index below its own) whose squared distance is strictly below the current
// worst, re-sorting its m-list with R's Shell sort.  One thread runs one
// location's walk; distances use __dadd_rn/__dmul_rn so no FMA contraction
// changes a bit, which makes neighbor indices and distances bit-exact with the
// reference, ties included.  The sort of u is a radix sort; when two u values
// are equal the sorted order would depend on R's Shell sort, so in that case the
// exact Shell-sort passes are replayed on the device instead (each gap's chains
// are independent insertion sorts, one thread per chain).
//
// The walk visits the whole diagonal strip |u - u_q| < sqrt(2) r of the u order
// (about 4 n r candidates per location), so mkNNIndxCB first runs a
// grid-bucketed search (grid_knn_kernel) that finds the same lists, and only
// the locations whose list could depend on the walk's order (equal keys, or a
// near-tie at the list's end) are walked.
//
// mkNNIndx (src/nn.cpp:63-111): exhaustive scan j = 0..i-1 per location with
// the reference's acceptance rule on the Euclidean distance.
//
// nn2 (the RANN::nn2 calls of R/spConjNNGP.R:158,311, R/generics.R:642):
// unconstrained exact kNN of prediction points against the training points on
// the same grid, ordered by (squared distance, index).
//
// mkUIndx (src/nn.cpp:25-56, src/util.cpp:115-185): a stable radix sort of the
// packed neighbor entries by neighbor id gives, for each location, the
// locations listing it in increasing order, and the entry positions give uiIndx.
#include <cuda_runtime.h>
#include <cub/cub.cuh>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#include "nngp_internal.h"

namespace {

// The neighbor lists hold non-negative distances (or +inf), whose IEEE bit patterns
// order exactly like signed 64-bit integers, so the lists keep the bit patterns and
// compare them on the integer pipe.  R's Shell sort on such keys:
__device__ void shell_sort_keys(long long *x, int *idx, int n) {
  int gap = 1;
  while (gap <= n / 9) gap = 3 * gap + 1;
  for (; gap > 0; gap /= 3) {
    for (int i = gap; i < n; i++) {
      const long long key = x[i];
      const int tag = idx[i];
      int j = i;
      while (j >= gap && x[j - gap] > key) {
        x[j] = x[j - gap];
        idx[j] = idx[j - gap];
        j -= gap;
      }
      x[j] = key;
      idx[j] = tag;
    }
  }
}

// Replaces the last (worst) entry of a sorted list by (key, tag) and re-sorts it exactly as
// R's rsort_with_index would.  While the list holds no equal keys and the new key equals none
// of them, every sort yields the same order, so a plain insertion is used; once a tie exists
// the Shell sort itself runs (it may reorder tied entries).
__device__ __forceinline__ void list_insert(long long *x, int *idx, int n, long long key, int tag, bool &ties) {
  if (!ties) {
    int j = n - 1;
    while (j > 0 && x[j - 1] > key) {
      x[j] = x[j - 1];
      idx[j] = idx[j - 1];
      j--;
    }
    if (j > 0 && x[j - 1] == key) {
      // undo the shifts and hand the list to the exact sort
      for (int t = j; t < n - 1; t++) {
        x[t] = x[t + 1];
        idx[t] = idx[t + 1];
      }
      ties = true;
    } else {
      x[j] = key;
      idx[j] = tag;
      return;
    }
  }
  x[n - 1] = key;
  idx[n - 1] = tag;
  shell_sort_keys(x, idx, n);
}

// Packed-list offset / length of location i (src/util.cpp:55-70).
__device__ __forceinline__ void nn_slot(int i, int m, int &off, int &cnt) {
  if (i == 0) {
    off = 0;
    cnt = 0;
  } else if (i < m) {
    off = (int)((double)i / 2 * (i - 1));
    cnt = i;
  } else {
    off = (int)((double)m / 2 * (m - 1) + (double)((i - m) * m));
    cnt = m;
  }
}

__global__ void ukey_kernel(const double *__restrict__ cm, int n, double *__restrict__ u, int *__restrict__ idx) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    u[i] = __dadd_rn(cm[i], cm[n + i]);
    idx[i] = i;
  }
}

__global__ void tie_kernel(const double *__restrict__ us, int n, int *__restrict__ flag) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) {
    const double a = us[k];
    if (a != a || (k + 1 < n && a == us[k + 1])) atomicOr(flag, 1);
  }
}

// R's comparison for rsort_with_index on arbitrary doubles: NaN sorts last.
__device__ __forceinline__ bool gt_nan_last(double a, double b) {
  const bool na = isnan(a), nb = isnan(b);
  if (na && nb) return false;
  if (na) return true;
  if (nb) return false;
  return a > b;
}

// One gap pass of the Shell sort: thread c owns the chain c, c+h, c+2h, ...
__global__ void shell_pass_kernel(double *__restrict__ u, int *__restrict__ idx, int n, int h) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= h) return;
  for (int i = c + h; i < n; i += h) {
    const double key = u[i];
    const int tag = idx[i];
    int j = i;
    while (j >= h && gt_nan_last(u[j - h], key)) {
      u[j] = u[j - h];
      idx[j] = idx[j - h];
      j -= h;
    }
    u[j] = key;
    idx[j] = tag;
  }
}

__global__ void gather_sorted_kernel(const double *__restrict__ cm, int n, const int *__restrict__ sidx,
                                     double *__restrict__ xs, double *__restrict__ ys, float4 *__restrict__ sf,
                                     double cx, double cy) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) {
    const int j = sidx[s];
    const double x = cm[j], y = cm[n + j];
    xs[s] = x;
    ys[s] = y;
    if (sf) sf[s] = make_float4((float)(x - cx), (float)(y - cy), __int_as_float(j), 0.f);
  }
}

// Extent of the coordinates: out = (min x, max x, min y, max y) as ordered-integer keys.
__device__ __forceinline__ unsigned long long dkey(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double dval(unsigned long long k) {
  return __longlong_as_double((long long)((k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k));
}
__global__ void extent_kernel(const double *__restrict__ cm, int n, unsigned long long *__restrict__ out) {
  unsigned long long mnx = ~0ull, mxx = 0, mny = ~0ull, mxy = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const unsigned long long kx = dkey(cm[i]), ky = dkey(cm[n + i]);
    mnx = min(mnx, kx);
    mxx = max(mxx, kx);
    mny = min(mny, ky);
    mxy = max(mxy, ky);
  }
  // warp reduction first: one set of atomics per warp instead of per thread
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mnx = min(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
    mxx = max(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
    mny = min(mny, __shfl_xor_sync(0xffffffffu, mny, o));
    mxy = max(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&out[0], mnx);
    atomicMax(&out[1], mxx);
    atomicMin(&out[2], mny);
    atomicMax(&out[3], mxy);
  }
}

// Error bounds of the float pre-filter (unit roundoff u = 2^-24, FP64 e = 2^-53):
// coordinates are stored as x' = fl32(fl64(x - cx)); with S the largest |x - cx|, |y - cy|
// and M the largest |x|, |y|:
//   |fl32(x'_j - x'_q) - (x_j - x_q)| <= 5 u S                          (Ex)
//   |fl32(fx + fy) - du_ref|            <= 15 u S + 12 e M               (Eu)
// where du_ref is the reference's FP64 ((x_q + y_q) - x_j) - y_j up to sign.
struct FilterConsts {
  float ex, eu;
};

// Thresholds derived from the current worst squared distance W (rare: only on inserts).
struct FilterThr {
  float p0, p1, ins;  // |fu| <= p0: surely not pruned; |fu| > p1: surely pruned; lb >= ins: surely not inserted
};
__device__ __forceinline__ FilterThr make_thr(double W, const FilterConsts &fc) {
  FilterThr t;
  const double e64 = 1.1102230246251565e-16;
  const float hi = __double2float_ru(2.0 * W * (1.0 + 4 * e64));
  const float lo = __double2float_rd(2.0 * W * (1.0 - 4 * e64));
  t.p1 = __fadd_ru(__fsqrt_ru(hi), fc.eu);
  t.p0 = __fsub_rd(__fsqrt_rd(lo), fc.eu);
  t.ins = __double2float_ru(W * (1.0 + 8 * e64));
  return t;
}
// Lower bound (rounded down) of the candidate's true squared distance.
__device__ __forceinline__ float lower_de(float fx, float fy, const FilterConsts &fc) {
  const float ax = fmaxf(__fsub_rd(fabsf(fx), fc.ex), 0.f);
  const float ay = fmaxf(__fsub_rd(fabsf(fy), fc.ex), 0.f);
  return __fadd_rd(__fmul_rd(ax, ax), __fmul_rd(ay, ay));
}

// Code-book search for the location at sorted position s.  Each candidate is first
// classified in float with rigorous error bounds (surely pruned / surely kept / surely
// not inserted); only candidates the bounds cannot decide are evaluated with the
// reference's exact FP64 arithmetic, so every decision equals the reference's.
__global__ void __launch_bounds__(128) cb_kernel(int n, int m, const double *__restrict__ xs,
                                                 const double *__restrict__ ys, const float4 *__restrict__ sf,
                                                 FilterConsts fc, int *__restrict__ nnIndx,
                                                 double *__restrict__ nnDist, int *__restrict__ nnLU,
                                                 const int *__restrict__ slist, int nwork) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nwork) return;
  const int s = slist ? slist[w] : w;  // sorted position (all of them, or the listed ones)
  const float4 me = sf[s];
  const int q = __float_as_int(me.z);
  int off, cnt;
  nn_slot(q, m, off, cnt);
  nnLU[q] = off;
  nnLU[n + q] = cnt;
  if (cnt == 0) return;
  long long kl[NNGP_MAX_M_SEARCH];
  int il[NNGP_MAX_M_SEARCH];
  for (int k = 0; k < cnt; k++) {
    kl[k] = 0x7ff0000000000000ll;  // +inf
    il[k] = 0;
  }
  // the +inf fillers are identical (key, tag) pairs, so their mutual order never shows
  bool ties = false;
  double worst = __longlong_as_double(0x7ff0000000000000ll);
  FilterThr thr = make_thr(worst, fc);
  const double qx = xs[s], qy = ys[s];
  const double qu = __dadd_rn(qx, qy);
  int lo = s, hi = s;
  bool down = true, up = true;
  // one step of the walk at sorted position t (c = sf[t]); returns false when the direction
  // stops
  auto visit = [&](int t, const float4 c) -> bool {
    const float fx = __fsub_rn(c.x, me.x), fy = __fsub_rn(c.y, me.y);
    const float fu = fabsf(__fadd_rn(fx, fy));
    if (fu > thr.p1) return false;  // (u_q - u_j)^2 > 2 worst for sure
    if (!(fu <= thr.p0)) {          // undecided: the reference's own test
      const double du = __dadd_rn(__dadd_rn(qu, -xs[t]), -ys[t]);
      if (__dmul_rn(du, du) > 2.0 * worst) return false;
    }
    const int j = __float_as_int(c.z);
    if (j < q && !(lower_de(fx, fy, fc) >= thr.ins)) {
      const double dx = __dadd_rn(qx, -xs[t]), dy = __dadd_rn(qy, -ys[t]);
      const double de = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
      if (de < worst) {
        list_insert(kl, il, cnt, __double_as_longlong(de), j, ties);
        worst = __longlong_as_double(kl[cnt - 1]);
        if (ties) {
          // the exact sort is needed only while equal finite keys remain in the list
          bool any = false;
          for (int t = 1; t < cnt; t++) any |= (kl[t] == kl[t - 1] && kl[t] != 0x7ff0000000000000ll);
          ties = any;
        }
        thr = make_thr(worst, fc);
      }
    }
    return true;
  };
  // The walk alternates one step down and one step up, as the reference's does; each
  // step's decision needs its candidate, so the candidates of the next kWalkBatch steps in
  // both directions are loaded together (loads past a stop are simply not used) and the
  // steps then run in the reference's order on them.
  constexpr int kWalkBatch = 4;
  while (down || up) {
    float4 cd[kWalkBatch], cu[kWalkBatch];
#pragma unroll
    for (int k = 0; k < kWalkBatch; k++) {
      cd[k] = down ? sf[max(lo - 1 - k, 0)] : me;
      cu[k] = up ? sf[min(hi + 1 + k, n - 1)] : me;
    }
#pragma unroll
    for (int k = 0; k < kWalkBatch; k++) {
      if (lo == 0) down = false;
      if (hi == n - 1) up = false;
      if (down) {
        lo--;
        if (!visit(lo, cd[k])) down = false;
      }
      if (up) {
        hi++;
        if (!visit(hi, cu[k])) up = false;
      }
    }
  }
  for (int k = 0; k < cnt; k++) {
    nnIndx[off + k] = il[k];
    nnDist[off + k] = __dsqrt_rn(__longlong_as_double(kl[k]));
  }
}

// ------------------------------------------------------------ grid-bucketed search
// The code-book walk above visits every location of a diagonal strip of the u order (about
// 4 n r candidates for a neighbor radius r), so the primary search is a uniform grid instead:
// location q scans rings of cells around its own, outward, keeping the m smallest squared
// distances of predecessors (j < q; each cell lists its locations by increasing index, so
// the scan of a cell stops at the first j >= q), and stops once every unvisited cell is
// farther than the current m-th distance.  Distances use the reference's FP64 expression.
// Without ties this gives the reference's list -- the walk's stopping rule is exact, so the
// reference keeps the m smallest keys, sorted -- and a query is handed to the walk when its
// result could depend on the walk's order: two equal keys met, or the best key left out
// within 1e-13 (relative) of the list's last one (the walk's FP64 stopping test could then
// have decided differently from exact arithmetic).
struct GridGeom {
  double x0, y0, h, inv_h, slop;
  int nx, ny;
};
constexpr int kGridCellPoints = 3;  // mean locations per cell
constexpr int kGridBrute = 2048;    // locations q < kGridBrute scan their q predecessors directly

__device__ __forceinline__ int grid_coord(double v, double v0, double inv_h, int nc) {
  const int c = (int)floor((v - v0) * inv_h);
  return min(max(c, 0), nc - 1);
}

__global__ void grid_key_kernel(const double *__restrict__ cm, int n, GridGeom g, int *__restrict__ key,
                                int *__restrict__ val) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    key[i] = grid_coord(cm[n + i], g.y0, g.inv_h, g.ny) * g.nx + grid_coord(cm[i], g.x0, g.inv_h, g.nx);
    val[i] = i;
  }
}

// start[c] = first sorted position whose cell is >= c (c = 0 .. ncells)
__global__ void grid_start_kernel(const int *__restrict__ key, int n, int ncells, int *__restrict__ start) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int prev = p ? key[p - 1] : -1;
  for (int c = prev + 1; c <= key[p]; c++) start[c] = p;
  if (p == n - 1)
    for (int c = key[p] + 1; c <= ncells; c++) start[c] = n;
}

__global__ void grid_gather_kernel(const double *__restrict__ cm, int n, const int *__restrict__ val,
                                   double2 *__restrict__ gxy, int *__restrict__ gj) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n) {
    const int j = val[p];
    gxy[p] = make_double2(cm[j], cm[n + j]);
    gj[p] = j;
  }
}

__global__ void __launch_bounds__(128) grid_knn_kernel(int n, int m, const double *__restrict__ cm, GridGeom g,
                                                       const int *__restrict__ start,
                                                       const double2 *__restrict__ gxy, const int *__restrict__ gj,
                                                       int *__restrict__ nnIndx, double *__restrict__ nnDist,
                                                       int *__restrict__ nnLU, int *__restrict__ redo,
                                                       int *__restrict__ redo_count) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int off, cnt;
  nn_slot(q, m, off, cnt);
  nnLU[q] = off;
  nnLU[n + q] = cnt;
  if (cnt == 0) return;
  const double qx = cm[q], qy = cm[n + q];
  double kd[NNGP_MAX_M_SEARCH];
  int il[NNGP_MAX_M_SEARCH];
  const double inf = __longlong_as_double(0x7ff0000000000000ll);
  int have = 0;
  double worst = inf;  // the list's last key once it is full
  double next = inf;   // the smallest key left out (rejected or evicted)
  bool tie = false;
  auto consider = [&](int j, double xj, double yj) {
    const double dx = __dadd_rn(qx, -xj), dy = __dadd_rn(qy, -yj);
    const double de = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
    if (have == cnt && !(de < worst)) {
      tie |= de == worst;
      next = fmin(next, de);
      return;
    }
    int t;
    if (have == cnt) {
      next = fmin(next, kd[cnt - 1]);
      t = cnt - 1;
    } else {
      t = have++;
    }
    while (t > 0 && kd[t - 1] > de) {
      kd[t] = kd[t - 1];
      il[t] = il[t - 1];
      t--;
    }
    tie |= t > 0 && kd[t - 1] == de;
    kd[t] = de;
    il[t] = j;
    if (have == cnt) worst = kd[cnt - 1];
  };
  if (q < kGridBrute) {
    for (int j = 0; j < q; j++) consider(j, cm[j], cm[n + j]);
  } else {
    const int cx = grid_coord(qx, g.x0, g.inv_h, g.nx), cy = grid_coord(qy, g.y0, g.inv_h, g.ny);
    auto scan = [&](int c) {
      const int pe = start[c + 1];
      for (int p = start[c]; p < pe; p++) {
        const int j = gj[p];
        if (j >= q) break;
        const double2 v = gxy[p];
        consider(j, v.x, v.y);
      }
    };
    for (int k = 0;; k++) {
      // ring k: the cells at Chebyshev distance k, clipped to the grid
      const int ylo = max(cy - k, 0), yhi = min(cy + k, g.ny - 1);
      const int xlo = max(cx - k, 0), xhi = min(cx + k, g.nx - 1);
      for (int yy = ylo; yy <= yhi; yy++) {
        const int row = yy * g.nx;
        if (yy == cy - k || yy == cy + k) {
          for (int xx = xlo; xx <= xhi; xx++) scan(row + xx);
        } else {
          if (cx - k >= 0) scan(row + cx - k);
          if (k > 0 && cx + k < g.nx) scan(row + cx + k);
        }
      }
      // distance from q to the cells outside the searched box (none beyond a grid edge)
      double lb = inf;
      if (cx - k > 0) lb = fmin(lb, qx - (g.x0 + (cx - k) * g.h));
      if (cx + k < g.nx - 1) lb = fmin(lb, (g.x0 + (cx + k + 1) * g.h) - qx);
      if (cy - k > 0) lb = fmin(lb, qy - (g.y0 + (cy - k) * g.h));
      if (cy + k < g.ny - 1) lb = fmin(lb, (g.y0 + (cy + k + 1) * g.h) - qy);
      if (lb == inf) break;  // the box covers the grid
      if (have == cnt) {
        const double l = lb - g.slop;
        if (l > 0.0 && l * l > worst * (1.0 + 1e-12)) break;
      }
    }
  }
  if (tie || (have == cnt && next <= worst * (1.0 + 1e-13))) {
    redo[atomicAdd(redo_count, 1)] = q;
    return;
  }
  for (int k = 0; k < cnt; k++) {
    nnIndx[off + k] = il[k];
    nnDist[off + k] = __dsqrt_rn(kd[k]);
  }
}

// Exact k nearest training locations of one prediction point on the grid, ordered by
// (squared distance, index) like nn2_kernel: the order is total, so no case needs the walk.
// Points outside the training extent take the nearest edge cell; the box bound stays valid.
__global__ void __launch_bounds__(128) grid_nn2_kernel(int n0, const double *__restrict__ c0, int k, GridGeom g,
                                                       const int *__restrict__ start,
                                                       const double2 *__restrict__ gxy, const int *__restrict__ gj,
                                                       int *__restrict__ outIdx, double *__restrict__ outDist) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n0) return;
  const double qx = c0[q], qy = c0[n0 + q];
  double dl[NNGP_MAX_M_SEARCH];
  int il[NNGP_MAX_M_SEARCH];
  const double inf = __longlong_as_double(0x7ff0000000000000ll);
  int filled = 0;
  const int cx = grid_coord(qx, g.x0, g.inv_h, g.nx), cy = grid_coord(qy, g.y0, g.inv_h, g.ny);
  auto scan = [&](int c) {
    const int pe = start[c + 1];
    for (int p = start[c]; p < pe; p++) {
      const int j = gj[p];
      const double2 v = gxy[p];
      const double dx = __dadd_rn(qx, -v.x), dy = __dadd_rn(qy, -v.y);
      const double de = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
      if (filled == k && !(de < dl[k - 1] || (de == dl[k - 1] && j < il[k - 1]))) continue;
      int t = filled < k ? filled++ : k - 1;
      while (t > 0 && (dl[t - 1] > de || (dl[t - 1] == de && il[t - 1] > j))) {
        dl[t] = dl[t - 1];
        il[t] = il[t - 1];
        t--;
      }
      dl[t] = de;
      il[t] = j;
    }
  };
  for (int r = 0;; r++) {
    const int ylo = max(cy - r, 0), yhi = min(cy + r, g.ny - 1);
    const int xlo = max(cx - r, 0), xhi = min(cx + r, g.nx - 1);
    for (int yy = ylo; yy <= yhi; yy++) {
      const int row = yy * g.nx;
      if (yy == cy - r || yy == cy + r) {
        for (int xx = xlo; xx <= xhi; xx++) scan(row + xx);
      } else {
        if (cx - r >= 0) scan(row + cx - r);
        if (r > 0 && cx + r < g.nx) scan(row + cx + r);
      }
    }
    double lb = inf;
    if (cx - r > 0) lb = fmin(lb, qx - (g.x0 + (cx - r) * g.h));
    if (cx + r < g.nx - 1) lb = fmin(lb, (g.x0 + (cx + r + 1) * g.h) - qx);
    if (cy - r > 0) lb = fmin(lb, qy - (g.y0 + (cy - r) * g.h));
    if (cy + r < g.ny - 1) lb = fmin(lb, (g.y0 + (cy + r + 1) * g.h) - qy);
    if (lb == inf) break;
    if (filled == k) {
      const double l = lb - g.slop;
      if (l > 0.0 && l * l > dl[k - 1] * (1.0 + 1e-12)) break;
    }
  }
  for (int t = 0; t < k; t++) {
    outIdx[(size_t)t * n0 + q] = il[t];
    if (outDist) outDist[(size_t)t * n0 + q] = __dsqrt_rn(dl[t]);
  }
}

// pos_of[location] = sorted position (os: sorted position -> location)
__global__ void inverse_kernel(const int *__restrict__ os, int n, int *__restrict__ pos_of) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) pos_of[os[s]] = s;
}
__global__ void redo_list_kernel(const int *__restrict__ pos_of, const int *__restrict__ redo_q, int nredo,
                                 int *__restrict__ redo_s) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w < nredo) redo_s[w] = pos_of[redo_q[w]];
}

// Exhaustive ordered search, location i scans j = 0..i-1 on the Euclidean distance.
__global__ void __launch_bounds__(128) brute_kernel(int n, int m, const double *__restrict__ cm,
                                                    int *__restrict__ nnIndx, double *__restrict__ nnDist,
                                                    int *__restrict__ nnLU) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int off, cnt;
  nn_slot(i, m, off, cnt);
  nnLU[i] = off;
  nnLU[n + i] = cnt;
  if (cnt == 0) return;
  long long kl[NNGP_MAX_M_SEARCH];
  int il[NNGP_MAX_M_SEARCH];
  for (int k = 0; k < cnt; k++) {
    kl[k] = 0x7ff0000000000000ll;
    il[k] = 0;
  }
  bool ties = false;
  double worst = __longlong_as_double(0x7ff0000000000000ll);
  double thr = worst;  // squared distances above thr cannot beat worst
  const double xi = cm[i], yi = cm[n + i];
  for (int j = 0; j < i; j++) {
    const double dx = __dadd_rn(xi, -cm[j]), dy = __dadd_rn(yi, -cm[n + j]);
    const double de = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
    if (de > thr) continue;
    const double d = __dsqrt_rn(de);
    if (d < worst) {
      list_insert(kl, il, cnt, __double_as_longlong(d), j, ties);
      worst = __longlong_as_double(kl[cnt - 1]);
      if (ties) {
        bool any = false;
        for (int t = 1; t < cnt; t++) any |= (kl[t] == kl[t - 1] && kl[t] != 0x7ff0000000000000ll);
        ties = any;
      }
      thr = worst * worst * (1.0 + 1e-12);
    }
  }
  for (int k = 0; k < cnt; k++) {
    nnIndx[off + k] = il[k];
    nnDist[off + k] = __longlong_as_double(kl[k]);
  }
}

// Exact kNN of one prediction point against the u-sorted training points.
__global__ void __launch_bounds__(128) nn2_kernel(int n, const double *__restrict__ xs,
                                                  const double *__restrict__ ys, const int *__restrict__ os,
                                                  const double *__restrict__ us, int n0,
                                                  const double *__restrict__ c0, int k,
                                                  int *__restrict__ outIdx, double *__restrict__ outDist) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n0) return;
  const double qx = c0[q], qy = c0[n0 + q];
  const double qu = __dadd_rn(qx, qy);
  // first sorted position with u >= qu
  int a = 0, b = n;
  while (a < b) {
    const int mid = (a + b) >> 1;
    if (us[mid] < qu) a = mid + 1;
    else b = mid;
  }
  double dl[NNGP_MAX_M_SEARCH];
  int il[NNGP_MAX_M_SEARCH];
  int filled = 0;
  const double INF = __longlong_as_double(0x7ff0000000000000ll);
  double worst = INF;
  int lo = a - 1, hi = a;
  bool down = lo >= 0, up = hi < n;
  auto consider = [&](int s) -> bool {  // returns false when the direction is exhausted
    const double cx = xs[s], cy = ys[s];
    const double du = __dadd_rn(__dadd_rn(qu, -cx), -cy);
    const double dm = __dmul_rn(du, du);
    if (filled == k && dm > 2.0 * worst * (1.0 + 1e-12)) return false;
    const double dx = __dadd_rn(qx, -cx), dy = __dadd_rn(qy, -cy);
    const double de = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
    const int j = os[s];
    if (filled == k && !(de < dl[k - 1] || (de == dl[k - 1] && j < il[k - 1]))) return true;
    int pos = (filled < k) ? filled++ : k - 1;
    while (pos > 0 && (dl[pos - 1] > de || (dl[pos - 1] == de && il[pos - 1] > j))) {
      dl[pos] = dl[pos - 1];
      il[pos] = il[pos - 1];
      pos--;
    }
    dl[pos] = de;
    il[pos] = j;
    worst = (filled == k) ? dl[k - 1] : INF;
    return true;
  };
  while (down || up) {
    if (down) {
      if (!consider(lo)) down = false;
      else if (--lo < 0) down = false;
    }
    if (up) {
      if (!consider(hi)) up = false;
      else if (++hi >= n) up = false;
    }
  }
  for (int t = 0; t < k; t++) {
    outIdx[(size_t)t * n0 + q] = il[t];
    if (outDist) outDist[(size_t)t * n0 + q] = __dsqrt_rn(dl[t]);
  }
}

__global__ void entry_row_kernel(int n, const int *__restrict__ nnLU, int *__restrict__ erow) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int off = nnLU[r], cnt = nnLU[n + r];
  for (int k = 0; k < cnt; k++) erow[off + k] = r;
}

__global__ void iota_kernel(int *__restrict__ a, long cnt) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < cnt) a[t] = (int)t;
}

__global__ void count_kernel(const int *__restrict__ keys, long cnt, int *__restrict__ counts) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < cnt) atomicAdd(&counts[keys[t]], 1);
}

__global__ void uindx_fill_kernel(long cnt, const int *__restrict__ sortedEntry, const int *__restrict__ erow,
                                  const int *__restrict__ nnLU, int *__restrict__ uIndx, int *__restrict__ uiIndx) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < cnt) {
    const int e = sortedEntry[t];
    const int r = erow[e];
    uIndx[t] = r;
    uiIndx[t] = e - nnLU[r];
  }
}

__global__ void reverse_segments_kernel(int n, const int *__restrict__ ulu, int *__restrict__ uIndx,
                                        int *__restrict__ uiIndx) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  int a = ulu[c], b = ulu[c] + ulu[n + c] - 1;
  while (a < b) {
    int t = uIndx[a];
    uIndx[a] = uIndx[b];
    uIndx[b] = t;
    t = uiIndx[a];
    uiIndx[a] = uiIndx[b];
    uiIndx[b] = t;
    a++;
    b--;
  }
}

inline unsigned blocks(long cnt, int tpb) { return (unsigned)((cnt + tpb - 1) / tpb); }

// Extent of column-major device coordinates (min x, max x, min y, max y); synchronises.
int coord_extent(nngp_ctx *ctx, int n, const double *d_cm, double e[4]) {
  unsigned long long *ext;
  NNGP_ALLOC(ctx, ext, unsigned long long, S_MISC3, 4);
  const unsigned long long init[4] = {~0ull, 0ull, ~0ull, 0ull};
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(ext, init, sizeof init, cudaMemcpyHostToDevice, ctx->stream));
  extent_kernel<<<std::min<unsigned>(blocks(n, 256), 1024), 256, 0, ctx->stream>>>(d_cm, n, ext);
  NNGP_LAUNCH_CHECK(ctx);
  unsigned long long hk[4];
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(hk, ext, sizeof hk, cudaMemcpyDeviceToHost, ctx->stream));
  NNGP_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  for (int t = 0; t < 4; t++) {
    unsigned long long b = (hk[t] >> 63) ? (hk[t] & 0x7FFFFFFFFFFFFFFFull) : ~hk[t];
    memcpy(&e[t], &b, sizeof(double));
  }
  return NNGP_OK;
}

// Sorts (u, index) and builds the sorted SoA view.  coords: device, column-major.
int sorted_view(nngp_ctx *ctx, int n, const double *d_cm, double **xs, double **ys, int **os,
                double **us, bool exact_ties, float4 **sf, FilterConsts &fc) {
  double *u, *u2;
  int *idx, *idx2;
  NNGP_ALLOC(ctx, u, double, S_U, (size_t)n);
  NNGP_ALLOC(ctx, u2, double, S_V2, (size_t)n);
  NNGP_ALLOC(ctx, idx, int, S_IDX, (size_t)n);
  NNGP_ALLOC(ctx, idx2, int, S_IDX2, (size_t)n);
  ukey_kernel<<<blocks(n, 256), 256, 0, ctx->stream>>>(d_cm, n, u, idx);
  NNGP_LAUNCH_CHECK(ctx);
  size_t tmp = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tmp, u, u2, idx, idx2, n, 0, 64, ctx->stream);
  void *dtmp;
  NNGP_ALLOC(ctx, dtmp, unsigned char, S_SORT_TMP, tmp);
  NNGP_CUDA_TRY(ctx, cub::DeviceRadixSort::SortPairs(dtmp, tmp, u, u2, idx, idx2, n, 0, 64, ctx->stream));
  ctx->launches += 1;
  if (exact_ties) {
    int *flag;
    NNGP_ALLOC(ctx, flag, int, S_MISC, 1);
    NNGP_CUDA_TRY(ctx, cudaMemsetAsync(flag, 0, sizeof(int), ctx->stream));
    tie_kernel<<<blocks(n, 256), 256, 0, ctx->stream>>>(u2, n, flag);
    NNGP_LAUNCH_CHECK(ctx);
    int h_flag = 0;
    NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(&h_flag, flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    NNGP_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (h_flag) {
      // equal keys: replay R's Shell sort exactly on the unsorted (u, index) pairs
      std::vector<int> gaps;
      int gap = 1;
      while (gap <= n / 9) gap = 3 * gap + 1;
      for (; gap > 0; gap /= 3) gaps.push_back(gap);
      for (int h : gaps) {
        shell_pass_kernel<<<blocks(h, 128), 128, 0, ctx->stream>>>(u, idx, n, h);
        NNGP_LAUNCH_CHECK(ctx);
      }
      NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(u2, u, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
      NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(idx2, idx, sizeof(int) * n, cudaMemcpyDeviceToDevice, ctx->stream));
    }
  }
  // extent of the coordinates for the float pre-filter's error bounds
  double e[4];
  if (int st = coord_extent(ctx, n, d_cm, e)) return st;
  const double mnx = e[0], mxx = e[1], mny = e[2], mxy = e[3];
  const double cx = 0.5 * (mnx + mxx), cy = 0.5 * (mny + mxy);
  const double S = std::max(std::max(mxx - cx, cx - mnx), std::max(mxy - cy, cy - mny)) * (1.0 + 1e-12);
  const double M = std::max(std::max(std::fabs(mnx), std::fabs(mxx)), std::max(std::fabs(mny), std::fabs(mxy)));
  const double u32 = 5.9604644775390625e-08, e64 = 1.1102230246251565e-16;
  fc.ex = (float)((5 * u32 * S + 4 * e64 * M) * 1.001);
  fc.eu = (float)((15 * u32 * S + 12 * e64 * M) * 1.001);
  if (!std::isfinite(S) || !std::isfinite(M)) fc.ex = fc.eu = __builtin_inff();
  NNGP_ALLOC(ctx, *xs, double, S_XS, (size_t)n);
  NNGP_ALLOC(ctx, *ys, double, S_YS, (size_t)n);
  NNGP_ALLOC(ctx, *sf, float4, S_OS, (size_t)n);
  gather_sorted_kernel<<<blocks(n, 256), 256, 0, ctx->stream>>>(d_cm, n, idx2, *xs, *ys, *sf, cx, cy);
  NNGP_LAUNCH_CHECK(ctx);
  *os = idx2;
  if (us) *us = u2;
  return NNGP_OK;
}

// Builds the search grid over n locations (column-major device coordinates): cells of about
// kGridCellPoints locations, each listing its locations by increasing index (start: cell
// offsets, gxy / gj: coordinates and indices in cell order).  usable = false when the extent
// is degenerate or not finite (the caller runs the walk instead).
int build_grid(nngp_ctx *ctx, int n, const double *coords, GridGeom &g, int **start, double2 **gxy, int **gj,
               bool &usable) {
  double e[4];
  int st = coord_extent(ctx, n, coords, e);
  if (st) return st;
  const double W = e[1] - e[0], H = e[3] - e[2], span = std::max(W, H);
  usable = std::isfinite(W) && std::isfinite(H) && span > 0.0;
  if (!usable) return NNGP_OK;
  const double area = std::max(W, 1e-3 * span) * std::max(H, 1e-3 * span);
  g.h = std::sqrt(area * kGridCellPoints / n);
  for (;;) {
    g.nx = (int)std::min(W / g.h, 1e9) + 1;
    g.ny = (int)std::min(H / g.h, 1e9) + 1;
    if ((long long)g.nx * g.ny <= 4LL * n + 64) break;
    g.h *= 1.25;
  }
  g.x0 = e[0];
  g.y0 = e[2];
  g.inv_h = 1.0 / g.h;
  const double M = std::max(std::max(std::fabs(e[0]), std::fabs(e[1])), std::max(std::fabs(e[2]), std::fabs(e[3])));
  g.slop = 1e-7 * g.h + 1e-13 * M;  // rounding of the cell assignment and of the box edges
  const int ncells = g.nx * g.ny;
  int *key, *key2, *val, *val2;
  NNGP_ALLOC(ctx, key, int, S_GKEY, (size_t)n);
  NNGP_ALLOC(ctx, key2, int, S_GKEY2, (size_t)n);
  NNGP_ALLOC(ctx, val, int, S_GJ, (size_t)n);
  NNGP_ALLOC(ctx, val2, int, S_GJ2, (size_t)n);
  NNGP_ALLOC(ctx, *gxy, double2, S_GXY, (size_t)n);
  NNGP_ALLOC(ctx, *start, int, S_GSTART, (size_t)ncells + 1);
  grid_key_kernel<<<blocks(n, 256), 256, 0, ctx->stream>>>(coords, n, g, key, val);
  NNGP_LAUNCH_CHECK(ctx);
  int bits = 1;
  while ((1LL << bits) < ncells) bits++;
  size_t tmp = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tmp, key, key2, val, val2, n, 0, bits, ctx->stream);
  void *dtmp;
  NNGP_ALLOC(ctx, dtmp, unsigned char, S_SORT_TMP, tmp);
  NNGP_CUDA_TRY(ctx, cub::DeviceRadixSort::SortPairs(dtmp, tmp, key, key2, val, val2, n, 0, bits, ctx->stream));
  ctx->launches += 1;
  grid_start_kernel<<<blocks(n, 256), 256, 0, ctx->stream>>>(key2, n, ncells, *start);
  NNGP_LAUNCH_CHECK(ctx);
  grid_gather_kernel<<<blocks(n, 256), 256, 0, ctx->stream>>>(coords, n, val2, *gxy, val);
  NNGP_LAUNCH_CHECK(ctx);
  *gj = val;
  return NNGP_OK;
}

int check_nn_args(nngp_ctx *ctx, int n, int m) {
  if (!ctx) return NNGP_ERR_ARG;
  if (n < 1 || m < 1 || m > NNGP_MAX_M_SEARCH)
    return nngp_fail(ctx, NNGP_ERR_ARG, "n >= 1 and 1 <= m <= 64 required");
  if (nngp_nindx(n, m) < 0) return nngp_fail(ctx, NNGP_ERR_ARG, "n must be at least m");
  return NNGP_OK;
}

}  // namespace

extern "C" {

int nngp_mkNNIndxCB_dev(nngp_ctx *ctx, int n, int m, const double *coords, int *nnIndx,
                        double *nnDist, int *nnIndxLU) {
  int st = check_nn_args(ctx, n, m);
  if (st) return st;
  cudaSetDevice(ctx->device);
  int *redo_q = nullptr;
  int nredo = n;  // every location by the walk unless the grid runs
  if (n > kGridBrute) {
    GridGeom g;
    int *start, *gj;
    double2 *gxy;
    bool usable = false;
    if ((st = build_grid(ctx, n, coords, g, &start, &gxy, &gj, usable))) return st;
    if (usable) {
      NNGP_ALLOC(ctx, redo_q, int, S_GREDO, (size_t)n + 1);
      int *cnt_d = redo_q + n;
      NNGP_CUDA_TRY(ctx, cudaMemsetAsync(cnt_d, 0, sizeof(int), ctx->stream));
      grid_knn_kernel<<<blocks(n, 128), 128, 0, ctx->stream>>>(n, m, coords, g, start, gxy, gj, nnIndx, nnDist,
                                                                 nnIndxLU, redo_q, cnt_d);
      NNGP_LAUNCH_CHECK(ctx);
      NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(&nredo, cnt_d, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
      NNGP_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    }
  }
  if (nredo > 0) {
    // the code-book walk: every location (small or degenerate inputs), or the listed ones
    double *xs, *ys;
    int *os;
    float4 *sf;
    FilterConsts fc;
    if ((st = sorted_view(ctx, n, coords, &xs, &ys, &os, nullptr, true, &sf, fc))) return st;
    int *redo_s = nullptr;
    if (redo_q) {
      int *pos_of;
      NNGP_ALLOC(ctx, pos_of, int, S_GKEY, (size_t)n);
      NNGP_ALLOC(ctx, redo_s, int, S_GKEY2, (size_t)nredo);
      inverse_kernel<<<blocks(n, 256), 256, 0, ctx->stream>>>(os, n, pos_of);
      NNGP_LAUNCH_CHECK(ctx);
      redo_list_kernel<<<blocks(nredo, 256), 256, 0, ctx->stream>>>(pos_of, redo_q, nredo, redo_s);
      NNGP_LAUNCH_CHECK(ctx);
    }
    cb_kernel<<<blocks(nredo, 128), 128, 0, ctx->stream>>>(n, m, xs, ys, sf, fc, nnIndx, nnDist, nnIndxLU, redo_s,
                                                           nredo);
    NNGP_LAUNCH_CHECK(ctx);
  }
  NNGP_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return NNGP_OK;
}

int nngp_mkNNIndxCB(nngp_ctx *ctx, int n, int m, const double *coords, int *nnIndx,
                    double *nnDist, int *nnIndxLU) {
  int st = check_nn_args(ctx, n, m);
  if (st) return st;
  cudaSetDevice(ctx->device);
  const int64_t nI = nngp_nindx(n, m);
  double *cm, *dd;
  int *di, *dlu;
  NNGP_ALLOC(ctx, cm, double, S_COORDS0, 2 * (size_t)n);
  NNGP_ALLOC(ctx, di, int, S_NNINDX, (size_t)(nI > 0 ? nI : 1));
  NNGP_ALLOC(ctx, dd, double, S_NNDIST, (size_t)(nI > 0 ? nI : 1));
  NNGP_ALLOC(ctx, dlu, int, S_NNLU, 2 * (size_t)n);
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(cm, coords, sizeof(double) * 2 * n, cudaMemcpyHostToDevice, ctx->stream));
  if ((st = nngp_mkNNIndxCB_dev(ctx, n, m, cm, di, dd, dlu))) return st;
  if (nI > 0) {
    NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(nnIndx, di, sizeof(int) * nI, cudaMemcpyDeviceToHost, ctx->stream));
    NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(nnDist, dd, sizeof(double) * nI, cudaMemcpyDeviceToHost, ctx->stream));
  }
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(nnIndxLU, dlu, sizeof(int) * 2 * n, cudaMemcpyDeviceToHost, ctx->stream));
  NNGP_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return NNGP_OK;
}

int nngp_mkNNIndx(nngp_ctx *ctx, int n, int m, const double *coords, int *nnIndx,
                  double *nnDist, int *nnIndxLU) {
  int st = check_nn_args(ctx, n, m);
  if (st) return st;
  cudaSetDevice(ctx->device);
  const int64_t nI = nngp_nindx(n, m);
  double *cm, *dd;
  int *di, *dlu;
  NNGP_ALLOC(ctx, cm, double, S_COORDS0, 2 * (size_t)n);
  NNGP_ALLOC(ctx, di, int, S_NNINDX, (size_t)(nI > 0 ? nI : 1));
  NNGP_ALLOC(ctx, dd, double, S_NNDIST, (size_t)(nI > 0 ? nI : 1));
  NNGP_ALLOC(ctx, dlu, int, S_NNLU, 2 * (size_t)n);
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(cm, coords, sizeof(double) * 2 * n, cudaMemcpyHostToDevice, ctx->stream));
  brute_kernel<<<blocks(n, 128), 128, 0, ctx->stream>>>(n, m, cm, di, dd, dlu);
  NNGP_LAUNCH_CHECK(ctx);
  if (nI > 0) {
    NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(nnIndx, di, sizeof(int) * nI, cudaMemcpyDeviceToHost, ctx->stream));
    NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(nnDist, dd, sizeof(double) * nI, cudaMemcpyDeviceToHost, ctx->stream));
  }
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(nnIndxLU, dlu, sizeof(int) * 2 * n, cudaMemcpyDeviceToHost, ctx->stream));
  NNGP_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return NNGP_OK;
}

int nngp_nn2_dev(nngp_ctx *ctx, int n, const double *coords, int n0, const double *coords0, int k,
                 int *nnIdx, double *nnDist) {
  if (!ctx) return NNGP_ERR_ARG;
  if (n < 1 || n0 < 0 || k < 1 || k > NNGP_MAX_M_SEARCH || k > n)
    return nngp_fail(ctx, NNGP_ERR_ARG, "nn2 needs 1 <= k <= min(n, 64)");
  if (n0 == 0) return NNGP_OK;
  cudaSetDevice(ctx->device);
  GridGeom g;
  int *start, *gj;
  double2 *gxy;
  bool usable = false;
  int st = build_grid(ctx, n, coords, g, &start, &gxy, &gj, usable);
  if (st) return st;
  if (usable) {
    grid_nn2_kernel<<<blocks(n0, 128), 128, 0, ctx->stream>>>(n0, coords0, k, g, start, gxy, gj, nnIdx, nnDist);
    NNGP_LAUNCH_CHECK(ctx);
    return NNGP_OK;
  }
  // degenerate extent (all training locations at one point): the u-order walk
  double *xs, *ys, *us;
  int *os;
  float4 *sf;
  FilterConsts fc;
  if ((st = sorted_view(ctx, n, coords, &xs, &ys, &os, &us, false, &sf, fc))) return st;
  nn2_kernel<<<blocks(n0, 128), 128, 0, ctx->stream>>>(n, xs, ys, os, us, n0, coords0, k, nnIdx, nnDist);
  NNGP_LAUNCH_CHECK(ctx);
  return NNGP_OK;
}

int nngp_nn2(nngp_ctx *ctx, int n, const double *coords, int n0, const double *coords0, int k,
             int *nnIdx, double *nnDist) {
  if (!ctx) return NNGP_ERR_ARG;
  if (n < 1 || n0 < 0 || k < 1 || k > NNGP_MAX_M_SEARCH || k > n)
    return nngp_fail(ctx, NNGP_ERR_ARG, "nn2 needs 1 <= k <= min(n, 64)");
  if (n0 == 0) return NNGP_OK;
  cudaSetDevice(ctx->device);
  double *cm, *c0, *dd;
  int *di;
  NNGP_ALLOC(ctx, cm, double, S_COORDS0, 2 * (size_t)n);
  NNGP_ALLOC(ctx, c0, double, S_COORDS, 2 * (size_t)n0);
  NNGP_ALLOC(ctx, di, int, S_NNINDX0, (size_t)n0 * k);
  NNGP_ALLOC(ctx, dd, double, S_OUT0, (size_t)n0 * k);
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(cm, coords, sizeof(double) * 2 * n, cudaMemcpyHostToDevice, ctx->stream));
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(c0, coords0, sizeof(double) * 2 * n0, cudaMemcpyHostToDevice, ctx->stream));
  int st = nngp_nn2_dev(ctx, n, cm, n0, c0, k, di, dd);
  if (st) return st;
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(nnIdx, di, sizeof(int) * n0 * k, cudaMemcpyDeviceToHost, ctx->stream));
  if (nnDist)
    NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(nnDist, dd, sizeof(double) * n0 * k, cudaMemcpyDeviceToHost, ctx->stream));
  NNGP_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return NNGP_OK;
}

int nngp_mkUIndx(nngp_ctx *ctx, int n, int m, const int *nnIndx, int *uIndx, int *uIndxLU,
                 int *uiIndx, const int *nnIndxLU, int searchType) {
  int st = check_nn_args(ctx, n, m);
  if (st) return st;
  cudaSetDevice(ctx->device);
  const long nI = (long)nngp_nindx(n, m);
  int *keys, *keys2, *ent, *ent2, *erow, *dlu, *ulu, *du, *dui;
  NNGP_ALLOC(ctx, keys, int, S_NNINDX, (size_t)(nI > 0 ? nI : 1));
  NNGP_ALLOC(ctx, keys2, int, S_IDX, (size_t)(nI > 0 ? nI : 1));
  NNGP_ALLOC(ctx, ent, int, S_IDX2, (size_t)(nI > 0 ? nI : 1));
  NNGP_ALLOC(ctx, ent2, int, S_MISC2, (size_t)(nI > 0 ? nI : 1));
  NNGP_ALLOC(ctx, erow, int, S_MISC3, (size_t)(nI > 0 ? nI : 1));
  NNGP_ALLOC(ctx, dlu, int, S_NNLU, 2 * (size_t)n);
  NNGP_ALLOC(ctx, ulu, int, S_OUT1, 2 * (size_t)n);
  NNGP_ALLOC(ctx, du, int, S_OUT2, (size_t)(nI > 0 ? nI : 1));
  NNGP_ALLOC(ctx, dui, int, S_OUT3, (size_t)(nI > 0 ? nI : 1));
  if (nI > 0) NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(keys, nnIndx, sizeof(int) * nI, cudaMemcpyHostToDevice, ctx->stream));
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(dlu, nnIndxLU, sizeof(int) * 2 * n, cudaMemcpyHostToDevice, ctx->stream));
  NNGP_CUDA_TRY(ctx, cudaMemsetAsync(ulu + n, 0, sizeof(int) * n, ctx->stream));
  if (nI > 0) {
    entry_row_kernel<<<blocks(n, 256), 256, 0, ctx->stream>>>(n, dlu, erow);
    NNGP_LAUNCH_CHECK(ctx);
    iota_kernel<<<blocks(nI, 256), 256, 0, ctx->stream>>>(ent, nI);
    NNGP_LAUNCH_CHECK(ctx);
    count_kernel<<<blocks(nI, 256), 256, 0, ctx->stream>>>(keys, nI, ulu + n);
    NNGP_LAUNCH_CHECK(ctx);
    size_t tmp = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tmp, keys, keys2, ent, ent2, (int)nI, 0, 32, ctx->stream);
    size_t tmp2 = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tmp2, ulu + n, ulu, n, ctx->stream);
    void *dtmp;
    NNGP_ALLOC(ctx, dtmp, unsigned char, S_SORT_TMP, tmp > tmp2 ? tmp : tmp2);
    NNGP_CUDA_TRY(ctx, cub::DeviceRadixSort::SortPairs(dtmp, tmp, keys, keys2, ent, ent2, (int)nI, 0, 32, ctx->stream));
    NNGP_CUDA_TRY(ctx, cub::DeviceScan::ExclusiveSum(dtmp, tmp2, ulu + n, ulu, n, ctx->stream));
    ctx->launches += 2;
    uindx_fill_kernel<<<blocks(nI, 256), 256, 0, ctx->stream>>>(nI, ent2, erow, dlu, du, dui);
    NNGP_LAUNCH_CHECK(ctx);
    if (searchType == 1) {
      reverse_segments_kernel<<<blocks(n, 256), 256, 0, ctx->stream>>>(n, ulu, du, dui);
      NNGP_LAUNCH_CHECK(ctx);
    }
    NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(uIndx, du, sizeof(int) * nI, cudaMemcpyDeviceToHost, ctx->stream));
    NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(uiIndx, dui, sizeof(int) * nI, cudaMemcpyDeviceToHost, ctx->stream));
  } else {
    NNGP_CUDA_TRY(ctx, cudaMemsetAsync(ulu, 0, sizeof(int) * n, ctx->stream));
  }
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(uIndxLU, ulu, sizeof(int) * 2 * n, cudaMemcpyDeviceToHost, ctx->stream));
  NNGP_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return NNGP_OK;
}

}  // extern "C"
