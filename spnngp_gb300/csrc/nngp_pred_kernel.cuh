// Prediction-point neighborhood solves (instantiated in nngp_pred_inst_*.cu).
//
// One thread owns one (prediction point, parameter set) pair: it builds the m x m
// covariance of the point's m training neighbors and their covariance with the
// point, factors it (packed triangle in shared memory, as in the B/F pass) and
// solves w = C^-1 c, then
//   KIND_CONJ  (src/cNNGP.cpp:252-300): yhat = x0'b + w'(y_N - X_N b),
//              var = b* (u'V u + 1 + alpha - w'c) / (a* - 1), u = x0 - X_N'w;
//   KIND_RESP  (src/rNNGPPredict.cpp:139-183): one posterior-predictive draw
//              y0 = x0'beta_s + w'(y_N - X_N beta_s) + sqrt(s2 + t2 - w'c) z.
// FP32R builds and factors in float and refines w once with an FP64 residual.
#pragma once
#include <cuda_runtime.h>
#include <type_traits>
#include "nngp_internal.h"
#include "nngp_math.cuh"

#include "nngp_pred.h"

namespace nngp_pred {

template <int M>
__host__ __device__ constexpr int ptri_size() { return M * (M + 1) / 2; }
__host__ __device__ constexpr int ptri_at(int r, int c) { return r * (r + 1) / 2 + c; }

template <int M, bool R32>
constexpr int pred_tpb() {
  return R32 ? (M <= 16 ? 128 : 64) : (M <= 16 ? 64 : 32);
}

template <int M, bool R32, int KIND, int TPB>
__global__ void __launch_bounds__(TPB) pred_kernel(PredArgs a) {
  using T = typename std::conditional<R32, float, double>::type;
  constexpr int GEO = R32 ? 4 : 2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *tri = reinterpret_cast<T *>(smem_raw);
  T *geo = tri + (size_t)ptri_size<M>() * TPB;
  const int tid = threadIdx.x;
#define TRI_(r, c) tri[(size_t)ptri_at((r), (c)) * TPB + tid]
#define GEO_(k, q) geo[(size_t)((k) * GEO + (q)) * TPB + tid]
  const long total = (long)a.n0 * a.npar;
  const long w = (long)blockIdx.x * TPB + tid;
  const bool active = w < total;
  // conjugate: consecutive threads share a grid point; response: consecutive threads share a point
  int i = 0, k = 0;
  if (active) {
    if (KIND == KIND_CONJ) {
      k = (int)(w / a.n0);
      i = (int)(w % a.n0);
    } else {
      i = (int)(w / a.npar);
      k = (int)(w % a.npar);
    }
  }
  const int mi = active ? a.m : 0;
  const CovParams *cpp = a.par + k;
  const double s2d = active ? cpp->sigmaSq : 1.0, t2d = active ? cpp->tauSq : 0.0;
  const double qx = active ? a.c0[i] : 0.0, qy = active ? a.c0[a.n0 + i] : 0.0;
  int nb[M];
#pragma unroll
  for (int j = 0; j < M; j++) {
    nb[j] = 0;
    if (j < mi) {
      nb[j] = a.nn0[(size_t)j * a.n0 + i];
      const double2 q = reinterpret_cast<const double2 *>(a.xy)[nb[j]];
      if constexpr (R32) {
        const double dx = q.x - qx, dy = q.y - qy;
        const float hx = (float)dx, hy = (float)dy;
        GEO_(j, 0) = hx;
        GEO_(j, 1) = hy;
        GEO_(j, 2) = (float)(dx - (double)hx);
        GEO_(j, 3) = (float)(dy - (double)hy);
      } else {
        GEO_(j, 0) = q.x;
        GEO_(j, 1) = q.y;
      }
    }
  }
  const T s2 = (T)s2d, t2 = (T)t2d;
  const float phif = (float)cpp->phi;
  T cv[M];
#pragma unroll
  for (int r = 0; r < M; r++) {
    cv[r] = (T)0;
    if (r < mi) {
      if constexpr (R32) {
        const float hx = GEO_(r, 0), hy = GEO_(r, 1);
        cv[r] = s2 * nngp_cor_f(hx * hx + hy * hy, *cpp, phif);
#pragma unroll
        for (int c = 0; c <= r; c++) {
          float e;
          if (c == r) {
            e = s2 + t2;
          } else {
            const float ex = (GEO_(r, 0) - GEO_(c, 0)) + (GEO_(r, 2) - GEO_(c, 2));
            const float ey = (GEO_(r, 1) - GEO_(c, 1)) + (GEO_(r, 3) - GEO_(c, 3));
            e = s2 * nngp_cor_f(ex * ex + ey * ey, *cpp, phif);
          }
          TRI_(r, c) = e;
        }
      } else {
        const double xr = GEO_(r, 0), yr = GEO_(r, 1);
        const double ax = xr - qx, ay = yr - qy;
        cv[r] = s2d * nngp_cor_d(sqrt(ax * ax + ay * ay), *cpp);
#pragma unroll
        for (int c = 0; c <= r; c++) {
          const double bx = xr - GEO_(c, 0), by = yr - GEO_(c, 1);
          double e = s2d * nngp_cor_d(sqrt(bx * bx + by * by), *cpp);
          if (c == r) e += t2d;
          TRI_(r, c) = e;
        }
      }
    }
  }
  T invd[M], z[M];
  bool ok = true;
#pragma unroll
  for (int r = 0; r < M; r++) {
    invd[r] = (T)0;
    z[r] = (T)0;
    if (r < mi) {
      T row[M];
#pragma unroll
      for (int c = 0; c <= r; c++) {
        T s = TRI_(r, c);
#pragma unroll
        for (int q = 0; q < c; q++) s -= row[q] * ((c == r) ? row[q] : TRI_(c, q));
        if (c < r) {
          row[c] = s * invd[c];
        } else {
          ok = ok && (s > (T)0);
          const T dg = sqrt(s);
          row[r] = dg;
          invd[r] = (T)1 / dg;
        }
      }
      T zs = cv[r];
#pragma unroll
      for (int q = 0; q < r; q++) zs -= row[q] * z[q];
      z[r] = zs * invd[r];
#pragma unroll
      for (int c = 0; c <= r; c++) TRI_(r, c) = row[c];
    }
  }
  T bb[M];
#pragma unroll
  for (int q = M - 1; q >= 0; q--) {
    bb[q] = (T)0;
    if (q < mi) {
      bb[q] = z[q] * invd[q];
#pragma unroll
      for (int r = 0; r < q; r++) z[r] -= TRI_(q, r) * bb[q];
    }
  }
  double wd[M];
  if constexpr (R32) {
    double res[M];
#pragma unroll
    for (int r = 0; r < M; r++) res[r] = (r < mi) ? (double)cv[r] : 0.0;
#pragma unroll
    for (int r = 0; r < M; r++) {
      if (r < mi) {
#pragma unroll
        for (int c = 0; c <= r; c++) {
          float e;
          if (c == r) {
            e = s2 + t2;
          } else {
            const float ex = (GEO_(r, 0) - GEO_(c, 0)) + (GEO_(r, 2) - GEO_(c, 2));
            const float ey = (GEO_(r, 1) - GEO_(c, 1)) + (GEO_(r, 3) - GEO_(c, 3));
            e = s2 * nngp_cor_f(ex * ex + ey * ey, *cpp, phif);
          }
          res[r] = fma(-(double)e, (double)bb[c], res[r]);
          if (c < r) res[c] = fma(-(double)e, (double)bb[r], res[c]);
        }
      }
    }
    T wv[M];
#pragma unroll
    for (int r = 0; r < M; r++) {
      wv[r] = (T)0;
      if (r < mi) {
        T s = (T)res[r];
#pragma unroll
        for (int q = 0; q < r; q++) s -= TRI_(r, q) * wv[q];
        wv[r] = s * invd[r];
      }
    }
#pragma unroll
    for (int q = M - 1; q >= 0; q--) {
      wd[q] = 0.0;
      if (q < mi) {
        const T dk = wv[q] * invd[q];
#pragma unroll
        for (int r = 0; r < q; r++) wv[r] -= TRI_(q, r) * dk;
        wd[q] = (double)bb[q] + (double)dk;
      }
    }
  } else {
#pragma unroll
    for (int q = 0; q < M; q++) wd[q] = (double)bb[q];
  }
  if (!active) return;
  if (!ok) {
    if constexpr (!R32) {
      atomicMin(a.status, (1ull << 48) | (unsigned long long)i);
    } else {
      // the float factor failed: flag the pair through the status word's FP64 retry code
      atomicMin(a.status, (4ull << 48) | (unsigned long long)i);
    }
  }
  const int p = a.p, nv = p + 1;
  double wc = 0.0;
#pragma unroll
  for (int q = 0; q < M; q++)
    if (q < mi) wc = fma(wd[q], (double)cv[q], wc);
  const double *bk = a.beta + (size_t)k * p;
  double fit = 0.0;
  for (int j = 0; j < p; j++) fit += a.X0[(size_t)j * a.n0 + i] * bk[j];
  double dsum = 0.0;
#pragma unroll
  for (int q = 0; q < M; q++) {
    if (q < mi) {
      const double *vr = a.V + (size_t)nb[q] * nv;
      double xb = 0.0;
      for (int j = 0; j < p; j++) xb += vr[j] * bk[j];
      dsum = fma(wd[q], vr[p] - xb, dsum);
    }
  }
  if (KIND == KIND_CONJ) {
    a.out0[(size_t)k * a.n0 + i] = fit + dsum;
    double u[NNGP_MAX_NV];
    for (int j = 0; j < p; j++) {
      double s = 0.0;
#pragma unroll
      for (int q = 0; q < M; q++)
        if (q < mi) s = fma(a.V[(size_t)nb[q] * nv + j], wd[q], s);
      u[j] = a.X0[(size_t)j * a.n0 + i] - s;
    }
    const double *Vk = a.Vinv + (size_t)k * p * p;
    double uvu = 0.0;
    for (int r = 0; r < p; r++)
      for (int c = 0; c < p; c++) uvu += u[r] * ((c <= r) ? Vk[c * p + r] : Vk[r * p + c]) * u[c];
    const double aa = a.ab[2 * k], bbk = a.ab[2 * k + 1];
    a.out1[(size_t)k * a.n0 + i] = bbk * (uvu + 1.0 + t2d - wc) / (aa - 1.0);
  } else {
    const double zz = a.z[(size_t)i * a.npar + k];
    a.out0[(size_t)k * a.n0 + i] = fit + dsum + sqrt(s2d + t2d - wc) * zz;
  }
#undef TRI_
#undef GEO_
}

template <int M, bool R32, int KIND>
int launch_pred(nngp_ctx *ctx, const PredArgs &a) {
  constexpr int TPB = pred_tpb<M, R32>();
  using T = typename std::conditional<R32, float, double>::type;
  constexpr int GEO = R32 ? 4 : 2;
  const size_t smem = sizeof(T) * ((size_t)ptri_size<M>() + (size_t)GEO * M) * TPB;
  auto kern = pred_kernel<M, R32, KIND, TPB>;
  static bool configured[64] = {};  // the attribute is per device
  const int dev = ctx->device & 63;
  if (!configured[dev]) {
    NNGP_CUDA_TRY(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    configured[dev] = true;
  }
  const long total = (long)a.n0 * a.npar;
  if (total <= 0) return NNGP_OK;
  kern<<<(unsigned)((total + TPB - 1) / TPB), TPB, smem, ctx->stream>>>(a);
  NNGP_LAUNCH_CHECK(ctx);
  return NNGP_OK;
}

}  // namespace nngp_pred
