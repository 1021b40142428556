// Sequence initialisation: the displacement field of the next frame predicted
// from earlier frames (func/funPOR_GPR.m:1-99; main_ALDIC_Quadtree_v2.m:179-197
// calls it once for u and once for v with the last five frames).
//
// The work over the np nodes -- the snapshot mean, the nT x nT correlation
// matrix under the reference's trapezoid inner product, the POD modes, their
// coefficients and the prediction -- runs on the GPU in three passes (each a
// grid-stride pass with per-block partial sums added in a fixed order by one
// block, so results do not depend on scheduling).  The nT x nT eigenproblem
// (cyclic Jacobi) and the Gaussian-process regression of the nB mode
// coefficients over nT times run on the host: they are a handful of dense
// 5 x 5 operations.
//
// The regression restates the documented model of MATLAB's fitrgp(t, a,
// 'Basis','linear','FitMethod','exact','PredictMethod','exact',
// 'SigmaLowerBound',2e-5): a squared-exponential kernel, the linear basis
// profiled out, hyperparameters maximising the exact log marginal likelihood
// from the documented starting point, by Nelder-Mead on log-parameters.
// MATLAB's own optimiser is a closed toolbox routine and is not restated.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/staqdic.h"
#include "device_common.cuh"
#include "kernels.h"

namespace stdic {
namespace {

constexpr int kMaxT = 16;     // snapshots
constexpr int kMaxB = 8;      // modes
constexpr int kPartials = 512;

// trapezoid weight of node p among np (the reference's inner product, before
// its 0.1 / (np - 1) factor)
STDIC_DEV double trap_w(long long p, long long np) { return (p == 0 || p == np - 1) ? 0.5 : 1.0; }

// Pass 1: ave[p] = mean over the snapshots; partial sums of the upper
// triangle of the correlation matrix of the mean-free snapshots.
__global__ void __launch_bounds__(256) por_corr_kernel(const double* __restrict__ T, int nT, long long np,
                                                       double* __restrict__ ave, double* __restrict__ part) {
  __shared__ double red[32];
  const int npair = nT * (nT + 1) / 2;
  double acc[kMaxT * (kMaxT + 1) / 2];
  for (int q = 0; q < npair; ++q) acc[q] = 0.0;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < np; p += (long long)gridDim.x * blockDim.x) {
    double v[kMaxT];
    double s = 0;
    for (int t = 0; t < nT; ++t) { v[t] = T[t + (long long)nT * p]; s += v[t]; }
    const double a = s / nT;
    ave[p] = a;
    const double wgt = trap_w(p, np);
    for (int t = 0; t < nT; ++t) v[t] -= a;
    int q = 0;
    for (int k = 0; k < nT; ++k)
      for (int j = k; j < nT; ++j) acc[q++] += wgt * v[k] * v[j];
  }
  for (int q = 0; q < npair; ++q) {
    double x = acc[q];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t2 = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t2 += red[w];
      part[(long long)q * kPartials + blockIdx.x] = t2;
    }
  }
}

// Pass 2: fi[k][p] = sum_t fp[t][p] w[t][k] / sqrt(lambda_k) and partial sums
// of the mode coefficients a[t][k] = <fp_t, fi_k>.
__global__ void __launch_bounds__(256) por_modes_kernel(const double* __restrict__ T, const double* __restrict__ ave,
                                                        int nT, long long np, int nB, const double* __restrict__ wk,
                                                        double* __restrict__ fi, double* __restrict__ part) {
  __shared__ double red[32];
  __shared__ double W[kMaxT * kMaxB];
  for (int q = threadIdx.x; q < nT * nB; q += blockDim.x) W[q] = wk[q];
  __syncthreads();
  double acc[kMaxT * kMaxB];
  for (int q = 0; q < nT * nB; ++q) acc[q] = 0.0;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < np; p += (long long)gridDim.x * blockDim.x) {
    double v[kMaxT];
    const double a = ave[p];
    for (int t = 0; t < nT; ++t) v[t] = T[t + (long long)nT * p] - a;
    const double wgt = trap_w(p, np);
    for (int k = 0; k < nB; ++k) {
      double f = 0;
      for (int t = 0; t < nT; ++t) f += v[t] * W[t * nB + k];  // W holds w(t,k) / sqrt(lambda_k)
      fi[(long long)k * np + p] = f;
      for (int t = 0; t < nT; ++t) acc[t * nB + k] += wgt * v[t] * f;
    }
  }
  for (int q = 0; q < nT * nB; ++q) {
    double x = acc[q];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t2 = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t2 += red[w];
      part[(long long)q * kPartials + blockIdx.x] = t2;
    }
  }
}

// The partial sums of m quantities over nb blocks, in block order.
__global__ void por_total_kernel(const double* __restrict__ part, int m, int nb, double scale, double* __restrict__ out) {
  for (int q = threadIdx.x; q < m; q += blockDim.x) {
    double s = 0;
    for (int b = 0; b < nb; ++b) s += part[(long long)q * kPartials + b];
    out[q] = s * scale;
  }
}

// Pass 3: u_pred[t1][p] = sum_k ypred[t1][k] fi[k][p] + ave[p] (nT1 x np,
// column-major like MATLAB's u_pred).
__global__ void __launch_bounds__(256) por_predict_kernel(const double* __restrict__ fi, const double* __restrict__ ave,
                                                          long long np, int nB, const double* __restrict__ yp, int nT1,
                                                          double* __restrict__ out) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < np; p += (long long)gridDim.x * blockDim.x) {
    for (int t1 = 0; t1 < nT1; ++t1) {
      double s = 0;
      for (int k = 0; k < nB; ++k) s += yp[t1 * nB + k] * fi[(long long)k * np + p];
      out[t1 + (long long)nT1 * p] = s + ave[p];
    }
  }
}

// ---- host: eigenproblem and regression ---------------------------------------
// Cyclic Jacobi on a symmetric n x n matrix (row-major): eigenvalues in lam,
// eigenvectors in the columns of V, both sorted by decreasing eigenvalue.
void jacobi_eig(std::vector<double> A, int n, std::vector<double>& lam, std::vector<double>& V) {
  V.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) V[i * n + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0;
    for (int i = 0; i < n; ++i)
      for (int j = i + 1; j < n; ++j) off += A[i * n + j] * A[i * n + j];
    if (off < 1e-300) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A[p * n + q];
        if (std::fabs(apq) < 1e-300) continue;
        const double th = (A[q * n + q] - A[p * n + p]) / (2 * apq);
        const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1));
        const double c = 1 / std::sqrt(t * t + 1), s = t * c;
        for (int k = 0; k < n; ++k) {
          const double akp = A[k * n + p], akq = A[k * n + q];
          A[k * n + p] = c * akp - s * akq;
          A[k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          const double apk = A[p * n + k], aqk = A[q * n + k];
          A[p * n + k] = c * apk - s * aqk;
          A[q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double vkp = V[k * n + p], vkq = V[k * n + q];
          V[k * n + p] = c * vkp - s * vkq;
          V[k * n + q] = s * vkp + c * vkq;
        }
      }
  }
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return A[a * n + a] > A[b * n + b]; });
  lam.resize(n);
  std::vector<double> Vs((size_t)n * n);
  for (int j = 0; j < n; ++j) {
    lam[j] = A[order[j] * n + order[j]];
    for (int i = 0; i < n; ++i) Vs[i * n + j] = V[i * n + order[j]];
  }
  V.swap(Vs);
}

// Cholesky of an SPD n x n (row-major) into L; false when not positive definite.
bool cholesky(const std::vector<double>& K, int n, std::vector<double>& L) {
  L.assign((size_t)n * n, 0.0);
  for (int j = 0; j < n; ++j) {
    double d = K[j * n + j];
    for (int k = 0; k < j; ++k) d -= L[j * n + k] * L[j * n + k];
    if (!(d > 0)) return false;
    L[j * n + j] = std::sqrt(d);
    for (int i = j + 1; i < n; ++i) {
      double s = K[i * n + j];
      for (int k = 0; k < j; ++k) s -= L[i * n + k] * L[j * n + k];
      L[i * n + j] = s / L[j * n + j];
    }
  }
  return true;
}

// x = K^-1 b from its Cholesky factor
std::vector<double> chol_solve(const std::vector<double>& L, int n, std::vector<double> b) {
  for (int i = 0; i < n; ++i) {
    double s = b[i];
    for (int k = 0; k < i; ++k) s -= L[i * n + k] * b[k];
    b[i] = s / L[i * n + i];
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = b[i];
    for (int k = i + 1; k < n; ++k) s -= L[k * n + i] * b[k];
    b[i] = s / L[i * n + i];
  }
  return b;
}

constexpr double kSigmaLower = 2e-5;

struct Gp {
  std::vector<double> t, y;
  int n;
  // kernel matrix plus noise for log-parameters q = log(sl, sf, sigma - lower)
  std::vector<double> K(const double* q) const {
    const double sl = std::exp(q[0]), sf = std::exp(q[1]), sn = kSigmaLower + std::exp(q[2]);
    std::vector<double> k((size_t)n * n);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        const double d = t[i] - t[j];
        k[i * n + j] = sf * sf * std::exp(-0.5 * d * d / (sl * sl)) + (i == j ? sn * sn : 0.0);
      }
    return k;
  }
  // basis coefficients b = (H' K^-1 H)^-1 H' K^-1 y with H = [1 t]
  void beta(const std::vector<double>& L, double b[2]) const {
    std::vector<double> h1(n, 1.0), h2(t);
    const auto k1 = chol_solve(L, n, h1), k2 = chol_solve(L, n, h2), ky = chol_solve(L, n, y);
    double a11 = 0, a12 = 0, a22 = 0, r1 = 0, r2 = 0;
    for (int i = 0; i < n; ++i) {
      a11 += h1[i] * k1[i]; a12 += h1[i] * k2[i]; a22 += h2[i] * k2[i];
      r1 += h1[i] * ky[i]; r2 += h2[i] * ky[i];
    }
    const double det = a11 * a22 - a12 * a12;
    b[0] = (a22 * r1 - a12 * r2) / det;
    b[1] = (a11 * r2 - a12 * r1) / det;
  }
  double nll(const double* q) const {
    std::vector<double> L;
    if (!cholesky(K(q), n, L)) return 1e300;
    double b[2];
    beta(L, b);
    std::vector<double> r(n);
    for (int i = 0; i < n; ++i) r[i] = y[i] - b[0] - b[1] * t[i];
    const auto kr = chol_solve(L, n, r);
    double quad = 0, logdet = 0;
    for (int i = 0; i < n; ++i) { quad += r[i] * kr[i]; logdet += std::log(L[i * n + i]); }
    return 0.5 * quad + logdet + 0.5 * n * std::log(2 * M_PI);
  }
};

// Nelder-Mead (reflection 1, expansion 2, contraction 1/2, shrink 1/2) from
// the simplex x0, x0 + step e_k, in the order of decisions of the oracle's.
void nelder_mead(const Gp& g, double x[3]) {
  const int n = 3;
  double P[4][3], V[4];
  for (int i = 0; i <= n; ++i)
    for (int k = 0; k < n; ++k) P[i][k] = x[k] + (i == k + 1 ? 0.5 : 0.0);
  for (int i = 0; i <= n; ++i) V[i] = g.nll(P[i]);
  for (int it = 0; it < 2000; ++it) {
    int order[4] = {0, 1, 2, 3};
    std::stable_sort(order, order + 4, [&](int a, int b) { return V[a] < V[b]; });
    double Ps[4][3], Vs[4];
    for (int i = 0; i <= n; ++i) {
      Vs[i] = V[order[i]];
      for (int k = 0; k < n; ++k) Ps[i][k] = P[order[i]][k];
    }
    std::memcpy(P, Ps, sizeof P);
    std::memcpy(V, Vs, sizeof V);
    if (std::fabs(V[n] - V[0]) <= 1e-12 * (std::fabs(V[0]) + 1e-12)) break;
    double c[3], xr[3];
    for (int k = 0; k < n; ++k) c[k] = (P[0][k] + P[1][k] + P[2][k]) / n;
    for (int k = 0; k < n; ++k) xr[k] = c[k] + (c[k] - P[n][k]);
    const double fr = g.nll(xr);
    if (fr < V[0]) {
      double xe[3];
      for (int k = 0; k < n; ++k) xe[k] = c[k] + 2 * (c[k] - P[n][k]);
      const double fe = g.nll(xe);
      if (fe < fr) { std::memcpy(P[n], xe, sizeof xe); V[n] = fe; }
      else { std::memcpy(P[n], xr, sizeof xr); V[n] = fr; }
    } else if (fr < V[n - 1]) {
      std::memcpy(P[n], xr, sizeof xr);
      V[n] = fr;
    } else {
      double xc[3];
      if (fr >= V[n]) for (int k = 0; k < n; ++k) xc[k] = c[k] + 0.5 * (P[n][k] - c[k]);
      else for (int k = 0; k < n; ++k) xc[k] = c[k] + 0.5 * (xr[k] - c[k]);
      const double fc = g.nll(xc);
      if (fc < std::min(fr, V[n])) {
        std::memcpy(P[n], xc, sizeof xc);
        V[n] = fc;
      } else {
        for (int i = 1; i <= n; ++i) {
          for (int k = 0; k < n; ++k) P[i][k] = P[0][k] + 0.5 * (P[i][k] - P[0][k]);
          V[i] = g.nll(P[i]);
        }
      }
    }
  }
  int best = 0;
  for (int i = 1; i <= n; ++i)
    if (V[i] < V[best]) best = i;
  for (int k = 0; k < n; ++k) x[k] = P[best][k];
}

double sample_std(const std::vector<double>& v) {
  const int n = (int)v.size();
  if (n < 2) return 1.0;
  double m = 0;
  for (double x : v) m += x;
  m /= n;
  double s = 0;
  for (double x : v) s += (x - m) * (x - m);
  return std::sqrt(s / (n - 1));
}

// One mode: prediction and standard deviation of a new observation at tp.
void gpr(const std::vector<double>& t, const std::vector<double>& y, const double* tp, int nT1, double* mean,
         double* sd) {
  Gp g{t, y, (int)t.size()};
  const double st = sample_std(t), sy = sample_std(y);
  double q[3] = {std::log(st > 0 ? st : 1.0), std::log(sy > 0 ? sy / std::sqrt(2.0) : 1.0),
                 std::log(sy > 0 ? std::max(sy / std::sqrt(2.0) - kSigmaLower, 1e-12) : 1.0)};
  nelder_mead(g, q);
  const int n = g.n;
  const double sl = std::exp(q[0]), sf = std::exp(q[1]), sn = kSigmaLower + std::exp(q[2]);
  std::vector<double> L;
  if (!cholesky(g.K(q), n, L)) {
    for (int i = 0; i < nT1; ++i) { mean[i] = NAN; sd[i] = NAN; }
    return;
  }
  double b[2];
  g.beta(L, b);
  std::vector<double> r(n);
  for (int i = 0; i < n; ++i) r[i] = y[i] - b[0] - b[1] * t[i];
  const auto alpha = chol_solve(L, n, r);
  for (int i = 0; i < nT1; ++i) {
    std::vector<double> ks(n);
    double m = b[0] + b[1] * tp[i];
    for (int j = 0; j < n; ++j) {
      const double d = tp[i] - t[j];
      ks[j] = sf * sf * std::exp(-0.5 * d * d / (sl * sl));
      m += ks[j] * alpha[j];
    }
    const auto kk = chol_solve(L, n, ks);
    double v = sf * sf + sn * sn;
    for (int j = 0; j < n; ++j) v -= ks[j] * kk[j];
    mean[i] = m;
    sd[i] = std::sqrt(v > 0 ? v : 0.0);
  }
}

}  // namespace

size_t por_workspace_bytes(long long np, int nT, int nB) {
  (void)nT;
  return (size_t)(np * (1 + nB) + (long long)kMaxT * kMaxB * kPartials + 4096) * sizeof(double);
}

int por_gpr(const double* T, int nT, long long np, const double* t_train, const double* t_pre, int nT1, int nB,
            double* u_pred, double* alpha_out, double* beta_pod, double* beta_gpr, void* ws, cudaStream_t s,
            long long* launches, const char** err) {
  *err = nullptr;
  if (nT < 2 || nT > kMaxT || nB < 1 || nB > kMaxB || nB > nT || np < 2 || nT1 < 1 || nT1 > 256) {
    *err = "funPOR_GPR: 2 <= nT <= 16 snapshots, 1 <= nB <= min(8, nT) modes, at least 2 nodes, 1..256 times";
    return STDIC_E_ARG;
  }
  double* ave = (double*)ws;
  double* fi = ave + np;
  double* part = fi + (long long)nB * np;
  double* tot = part + (long long)kMaxT * kMaxB * kPartials;
  double* wk = tot + 1024;
  double* yp = wk + 1024;
  const int blocks = (int)std::min<long long>(kPartials, std::max<long long>(1, std::min<long long>(
                                                             (np + 255) / 256, 4ll * current_sm_count())));
  const int npair = nT * (nT + 1) / 2;
  const double scale = 0.1 / (double)(np - 1);
  cudaError_t e = cudaSuccess;
  por_corr_kernel<<<blocks, 256, 0, s>>>(T, nT, np, ave, part);
  por_total_kernel<<<1, 128, 0, s>>>(part, npair, blocks, scale, tot);
  *launches += 2;
  std::vector<double> ctri(npair);
  e = cudaMemcpyAsync(ctri.data(), tot, npair * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) { *err = cudaGetErrorString(e); return STDIC_E_CUDA; }
  std::vector<double> C((size_t)nT * nT);
  for (int k = 0, q = 0; k < nT; ++k)
    for (int j = k; j < nT; ++j, ++q) C[k * nT + j] = C[j * nT + k] = ctri[q];
  std::vector<double> lam, V;
  jacobi_eig(C, nT, lam, V);
  if (beta_pod)
    *beta_pod = nB + 1 < nT ? (std::log(lam[1]) - std::log(lam[nB + 1])) / nB : NAN;
  double sall = 0, sB = 0;
  for (int k = 0; k < nT; ++k) sall += lam[k];
  for (int k = 0; k < nB; ++k) sB += lam[k];
  if (alpha_out) *alpha_out = sB / sall;
  std::vector<double> W((size_t)nT * nB);
  for (int t = 0; t < nT; ++t)
    for (int k = 0; k < nB; ++k) W[t * nB + k] = V[t * nT + k] / std::sqrt(lam[k]);
  e = cudaMemcpyAsync(wk, W.data(), W.size() * sizeof(double), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) { *err = cudaGetErrorString(e); return STDIC_E_CUDA; }
  por_modes_kernel<<<blocks, 256, 0, s>>>(T, ave, nT, np, nB, wk, fi, part);
  por_total_kernel<<<1, 128, 0, s>>>(part, nT * nB, blocks, scale, tot);
  *launches += 2;
  std::vector<double> a((size_t)nT * nB);
  e = cudaMemcpyAsync(a.data(), tot, a.size() * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) { *err = cudaGetErrorString(e); return STDIC_E_CUDA; }
  std::vector<double> tt(t_train, t_train + nT), ypred((size_t)nT1 * nB), ysd((size_t)nT1 * nB);
  for (int k = 0; k < nB; ++k) {
    std::vector<double> yk(nT), mk(nT1), sk(nT1);
    for (int t = 0; t < nT; ++t) yk[t] = a[t * nB + k];
    gpr(tt, yk, t_pre, nT1, mk.data(), sk.data());
    for (int i = 0; i < nT1; ++i) { ypred[i * nB + k] = mk[i]; ysd[i * nB + k] = sk[i]; }
  }
  if (beta_gpr)
    for (int i = 0; i < nT1; ++i) {
      double sd = 0, ws2 = 0;
      for (int k = 0; k < nB; ++k) { sd += ysd[i * nB + k] * lam[k]; ws2 += std::fabs(ypred[i * nB + k]) * lam[k]; }
      beta_gpr[i] = sd / ws2;
    }
  e = cudaMemcpyAsync(yp, ypred.data(), ypred.size() * sizeof(double), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) { *err = cudaGetErrorString(e); return STDIC_E_CUDA; }
  por_predict_kernel<<<blocks, 256, 0, s>>>(fi, ave, np, nB, yp, nT1, u_pred);
  ++*launches;
  e = cudaGetLastError();
  if (e != cudaSuccess) { *err = cudaGetErrorString(e); return STDIC_E_CUDA; }
  return STDIC_OK;
}

}  // namespace stdic
