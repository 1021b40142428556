// Plain FP64 drop-in IC-GN: one CTA per subset (node), reproducing
//   func_quadtree/funICGNQuadtree.m:29-448   (6-DOF first pass, LocalICGNQuadtree)
//   func/funICGN_Subpb1.m:34-471            (2-DOF augmented-Lagrangian Subpb1)
// with the reference's mask logic (bwselect flood fills, window growth, the
// size-mismatch error of the 6-DOF pass) and result codes.  Per-pixel values
// (warped positions, interpolated g) are rounded exactly as the reference
// rounds them; only the order of the block-wide sums differs from a serial loop.
#include <algorithm>

#include "device_common.cuh"
#include "kernels.h"

namespace stdic {

namespace {

struct Frame64 {
  const double* __restrict__ f;
  const double* __restrict__ g;
  const uint8_t* __restrict__ mask;
  const double* __restrict__ dfdx;
  const double* __restrict__ dfdy;
  int W, H;
  STDIC_DEV double F(long long x1, long long y1) const { return __ldg(f + (y1 - 1) * W + (x1 - 1)); }
  STDIC_DEV double M(long long x1, long long y1) const {
    return (double)__ldg(mask + (y1 - 1) * W + (x1 - 1));
  }
  STDIC_DEV double GX(long long x1, long long y1) const {
    return __ldg(dfdx + (y1 - 4) * (long long)(W - 6) + (x1 - 4));
  }
  STDIC_DEV double GY(long long x1, long long y1) const {
    return __ldg(dfdy + (y1 - 4) * (long long)(W - 6) + (x1 - 4));
  }
};

// crops ImgRef(x1:x3,..), Df.DfDx(x1-3:x3-3,..) exist only for 4 <= x1, x3 <= W-3
STDIC_DEV bool crop_ok(const Frame64& fr, long long x1, long long x3, long long y1, long long y3) {
  return x1 >= 4 && x3 <= fr.W - 3 && y1 >= 4 && y3 <= fr.H - 3;
}
STDIC_DEV bool mask_crop_ok(const Frame64& fr, long long x1, long long x3, long long y1,
                            long long y3) {
  return x1 >= 1 && x3 <= fr.W && y1 >= 1 && y3 <= fr.H;
}

// mean and sqrt((n-1)*var) over |t| > 1e-10 (funICGNQuadtree.m:119-120), two
// passes like MATLAB's mean/var; var of one sample is 0, of none NaN.
STDIC_DEV void masked_stats(const double* t, int npx, double* scratch, double* mean_out,
                            double* bottom_out) {
  double v[2] = {0.0, 0.0};
  for (int p = threadIdx.x; p < npx; p += blockDim.x) {
    const double x = t[p];
    if (fabs(x) > 1e-10) { v[0] += x; v[1] += 1.0; }
  }
  block_sum<2>(v, scratch);
  const double cnt = v[1];
  const double mean = v[0] / cnt;
  double q[1] = {0.0};
  for (int p = threadIdx.x; p < npx; p += blockDim.x) {
    const double x = t[p];
    if (fabs(x) > 1e-10) { const double d = x - mean; q[0] += d * d; }
  }
  block_sum<1>(q, scratch);
  double var;
  if (cnt == 0) var = nan("");
  else if (cnt == 1) var = 0.0;
  else var = q[0] / (cnt - 1);
  *mean_out = mean;
  *bottom_out = sqrt((cnt - 1) * var);
}

// Any warped tile pixel outside [3, W-2] x [3, H-2] (funICGNQuadtree.m:154)
STDIC_DEV bool any_oob(const Frame64& fr, const double P[6], long long x0, long long y0,
                       long long x1, long long y1, int mx, int my) {
  // The warp is affine, so every pixel lies in the hull of the four corner
  // pixels; rounding moves a position by about 1e-12 px at these image
  // sizes.  Threads 0-3 evaluate one corner each, with the same operations as
  // the per-pixel test: a corner outside is a pixel outside (the answer), and
  // corners inside by more than 1e-6 px put every pixel inside.  Only a
  // corner within 1e-6 px of the border takes the test of every pixel.
  {
    int out = 0, near = 0;
    if (threadIdx.x < 4) {
      const int i = (threadIdx.x & 1) ? mx - 1 : 0, j = (threadIdx.x & 2) ? my - 1 : 0;
      double u22, v22;
      warp_exact(P, (double)(x1 + i - x0), (double)(y1 + j - y0), (double)x0, (double)y0, &u22, &v22);
      const double xl = 3, xh = (double)fr.W - 2, yl = 3, yh = (double)fr.H - 2;
      if (u22 < xl || u22 > xh || v22 < yl || v22 > yh) out = 1;
      else if (!(u22 >= xl + 1e-6 && u22 <= xh - 1e-6 && v22 >= yl + 1e-6 && v22 <= yh - 1e-6)) near = 1;
    }
    // (__syncthreads_or returns whether any thread's value is nonzero, not
    // their bitwise or: one barrier per question)
    if (__syncthreads_or(out)) return true;
    if (!__syncthreads_or(near)) return false;
  }
  int bad = 0;
  const int npx = mx * my;
  for (int p = threadIdx.x; p < npx; p += blockDim.x) {
    const int i = p % mx, j = p / mx;
    double u22, v22;
    warp_exact(P, (double)(x1 + i - x0), (double)(y1 + j - y0), (double)x0, (double)y0, &u22, &v22);
    if (u22 < 3 || u22 > (double)fr.W - 2 || v22 < 3 || v22 > (double)fr.H - 2) bad = 1;
  }
  return __syncthreads_or(bad) != 0;
}

struct Shared {
  double P[6];
  double Hm[36];
  double L[36];  // 6-DOF: Cholesky factor of Hm (when hm_spd)
  int hm_spd;
  double red[32 * 21];
  int ired[32];
  int flag;
  int done;
  int code;
};

}  // namespace

// 6-DOF: per-pixel terms of the iterations that stay fixed over a subset,
// kept in shared memory when the class's tiles leave room for them.  The
// values are those the iterations would otherwise recompute, with the same
// operations, so the results do not change.
struct PlainCache {
  int rf;  // (tempf - meanf) / bottomf per pixel (one FP64 division per pixel less per iteration)
  int jg;  // masked gradients gx s, gy s per pixel, and the tile's dx, dy offsets per column and row
};

// Largest tile side of a class (its tiles are square, side^2 <= npx_cap).
__host__ __device__ inline int plain_side_cap(int npx_cap) {
  int m = 1;
  while ((m + 1) * (m + 1) <= npx_cap) ++m;
  return m;
}

// Dynamic shared memory of the 6-DOF kernel: tempg, [rf], [gx s, gy s],
// [dx, dy offsets] (doubles), then four npx_cap-byte bitmaps.
__host__ __device__ inline size_t plain6_smem_bytes(int npx_cap, PlainCache c) {
  const size_t d = (size_t)npx_cap * (1 + (c.rf ? 1 : 0) + (c.jg ? 2 : 0)) +
                   (c.jg ? 2 * (size_t)plain_side_cap(npx_cap) : 0);
  return d * sizeof(double) + 4 * (size_t)npx_cap;
}

// ---------------------------------------------------------------------------
// 6-DOF first pass.  Dynamic shared memory: npx_cap doubles (tempg), the
// cached terms of PlainCache, then 4 npx_cap bytes (mask tile, bw_f, bw_g,
// scratch bitmap).
// ---------------------------------------------------------------------------
// One node on the whole CTA; npx_cap is the tile capacity of the CTA's
// dynamic shared memory (the grown tile of the largest subset of its class).
__device__ void plain6_node(const IcgnArgs& a, const int node, unsigned char* dsm, Shared& sh,
                            const int npx_cap, const PlainCache cc) {
  Frame64 fr{(const double*)a.f, (const double*)a.g, a.mask, (const double*)a.dfdx,
             (const double*)a.dfdy, a.W, a.H};
  double* tg = (double*)dsm;
  double* dp = tg + npx_cap;
  double* rf = nullptr;
  double *gxs = nullptr, *gys = nullptr, *dxl = nullptr, *dyl = nullptr;
  if (cc.rf) { rf = dp; dp += npx_cap; }
  if (cc.jg) {
    const int mc = plain_side_cap(npx_cap);
    gxs = dp; gys = dp + npx_cap; dxl = gys + npx_cap; dyl = dxl + mc;
    dp = dyl + mc;
  }
  uint8_t* mtile = (uint8_t*)dp;
  uint8_t* bwf = mtile + npx_cap;
  uint8_t* bwg = bwf + npx_cap;
  uint8_t* tmp = bwg + npx_cap;

  const double cx = a.coords[node], cy = a.coords[a.N + node];
  const long long x0 = llround(cx), y0 = llround(cy);
  int ws = a.ws_list ? a.ws_list[node] : a.ws_all;
  const int ws0 = ws;
  const double tol = a.tol;
  const double U0x = a.U0[2 * node], U0y = a.U0[2 * node + 1];

  auto finish = [&](int code, bool nan_out, const double* P, const double* Hm) {
    if (threadIdx.x == 0) {
      a.conv[node] = code;
      if (nan_out) {
        a.U[2 * node] = a.U[2 * node + 1] = nan("");
        for (int k = 0; k < 4; ++k) a.F[4 * node + k] = nan("");
      } else {
        a.U[2 * node] = P[4]; a.U[2 * node + 1] = P[5];
        for (int k = 0; k < 4; ++k) a.F[4 * node + k] = P[k];
      }
      if (a.Hpk) {
        int q = 0;
        for (int col = 0; col < 6; ++col)
          for (int row = col; row < 6; ++row)
            a.Hpk[(size_t)q++ * a.N + node] = (Hm && !nan_out) ? Hm[row * 6 + col] : 0.0;
      }
    }
  };

  long long x1 = x0 - ws / 2, x3 = x0 + ws / 2, y1 = y0 - ws / 2, y3 = y0 + ws / 2;
  // markCoordHoleStrain flag of LocalICGNQuadtree.m:112-123 (original window)
  bool crop_valid = (ws % 2 == 0) && ws <= a.ws_max && mask_crop_ok(fr, x1, x3, y1, y3);
  int cntf = 0, nanf = 0;
  if (crop_valid) {
    const int m = ws + 1;
    for (int p = threadIdx.x; p < m * m; p += blockDim.x) {
      const int i = p % m, j = p / m;
      const double t = fr.F(x1 + i, y1 + j) * fr.M(x1 + i, y1 + j);
      if (t != t) nanf = 1;
      if (t == 0) ++cntf;
    }
  }
  cntf = block_sum_int(cntf, sh.ired);
  nanf = __syncthreads_or(nanf);
  if (a.mark && threadIdx.x == 0) a.mark[node] = (!crop_valid || cntf > 0) ? 1 : 0;
  double P[6] = {0, 0, 0, 0, U0x, U0y};
  if (!crop_valid || !crop_ok(fr, x1, x3, y1, y3) || nanf) { finish(-1, true, P, nullptr); return; }
  const double npx0 = (double)((ws + 1) * (ws + 1));
  if (!((double)cntf < 0.4 * npx0)) { finish(kMaxIter + 2, false, P, nullptr); return; }
  if ((double)cntf > 0.0 * npx0) {
    ws = (int)grow_window(npx0, npx0 - (double)cntf, ws);
    x1 = x0 - ws / 2; x3 = x0 + ws / 2; y1 = y0 - ws / 2; y3 = y0 + ws / 2;
    if (!mask_crop_ok(fr, x1, x3, y1, y3) || !crop_ok(fr, x1, x3, y1, y3) ||
        (ws + 1) * (ws + 1) > npx_cap) {
      finish(-1, true, P, nullptr);
      return;
    }
  }
  const int m = ws + 1, npx = m * m;
  const int c = (ws + 1) / 2;
  bool has_masked = false;
  {
    int z = 0;
    for (int p = threadIdx.x; p < npx; p += blockDim.x) {
      const int i = p % m, j = p / m;
      const uint8_t mk = __ldg(fr.mask + (y1 + j - 1) * fr.W + (x1 + i - 1)) != 0;
      mtile[p] = mk;
      if (!mk) z = 1;
    }
    has_masked = __syncthreads_or(z) != 0;
  }
  if (has_masked) bwselect_block(mtile, bwf, m, m, c, c, 4);
  else {
    for (int p = threadIdx.x; p < npx; p += blockDim.x) bwf[p] = 1;
    __syncthreads();
  }
  if (cc.jg)
    for (int k = threadIdx.x; k < m; k += blockDim.x) {
      dxl[k] = (double)(x1 + k - x0);
      dyl[k] = (double)(y1 + k - y0);
    }
  // tempf (masked) is staged in tg for the statistics, then regenerated on the fly
  {
    double h[21];
#pragma unroll
    for (int k = 0; k < 21; ++k) h[k] = 0;
    for (int p = threadIdx.x; p < npx; p += blockDim.x) {
      const int i = p % m, j = p / m;
      const double s = (double)bwf[p];
      const double gx = fr.GX(x1 + i, y1 + j) * s, gy = fr.GY(x1 + i, y1 + j) * s;
      if (cc.jg) { gxs[p] = gx; gys[p] = gy; }
      tg[p] = fr.F(x1 + i, y1 + j) * fr.M(x1 + i, y1 + j) * s;
      const double dx = (double)(x1 + i - x0), dy = (double)(y1 + j - y0);
      const double J[6] = {dx * gx, dx * gy, dy * gx, dy * gy, gx, gy};
      int q = 0;
#pragma unroll
      for (int aa = 0; aa < 6; ++aa)
#pragma unroll
        for (int bb = aa; bb < 6; ++bb) h[q++] += J[aa] * J[bb];
    }
    block_sum<21>(h, sh.red);
    if (threadIdx.x == 0) {
      int q = 0;
      for (int aa = 0; aa < 6; ++aa)
        for (int bb = aa; bb < 6; ++bb) { sh.Hm[aa * 6 + bb] = h[q]; sh.Hm[bb * 6 + aa] = h[q]; ++q; }
      // H is fixed over the iterations: its Cholesky factor is formed once
      // (mldivide's factorisation of the same matrix on every iteration)
      sh.hm_spd = chol6_factor(sh.Hm, sh.L) ? 1 : 0;
    }
  }
  double meanf, bottomf;
  masked_stats(tg, npx, sh.red, &meanf, &bottomf);
  double sabs;
  {
    double v[1] = {0};
    for (int p = threadIdx.x; p < npx; p += blockDim.x) {
      v[0] += fabs(tg[p]);
      // each thread keeps the f side of its own pixels' residuals
      if (cc.rf) rf[p] = (tg[p] - meanf) / bottomf;
    }
    block_sum<1>(v, sh.red);
    sabs = v[0];
  }

  double normNew = 1, normAbs = 1, normInit = 0;
  int step = 0;
  int cg = 0;  // sum(tempg_BW2) of the last iteration
  int code = 0;
  while (step <= kMaxIter && normNew > tol && normAbs > tol) {
    ++step;
    if (step > 1 && (double)cntf > 0.0 * npx0) {
      const double r = sqrt((double)((ws0 + 1) * (ws0 + 1)) / (double)cg) * ws / 2;
      if (!isfinite(r)) { code = -1; break; }
      const int nws = 2 * (int)ceil(r);
      if (nws != ws) {
        const long long nx1 = x0 - nws / 2, nx3 = x0 + nws / 2, ny1 = y0 - nws / 2, ny3 = y0 + nws / 2;
        if (!mask_crop_ok(fr, nx1, nx3, ny1, ny3)) { code = -1; break; }
        if (any_oob(fr, P, x0, y0, nx1, ny1, nws + 1, nws + 1)) { normNew = 1e6; break; }
        code = -1;  // tempf and tempg sizes disagree: MATLAB throws
        break;
      }
    }
    if (any_oob(fr, P, x0, y0, x1, y1, m, m)) { normNew = 1e6; break; }
    int zg = 0, nang = 0;
    for (int p = threadIdx.x; p < npx; p += blockDim.x) {
      const int i = p % m, j = p / m;
      double u22, v22;
      const double dxp = cc.jg ? dxl[i] : (double)(x1 + i - x0);
      const double dyp = cc.jg ? dyl[j] : (double)(y1 + j - y0);
      warp_exact(P, dxp, dyp, (double)x0, (double)y0, &u22, &v22);
      const double t = ba_cubic_exact(fr.g, fr.W, fr.H, v22, u22);
      tg[p] = t;
      if (t != t) nang = 1;
      if (t == 0) ++zg;
    }
    zg = block_sum_int(zg, sh.ired);
    if (__syncthreads_or(nang)) { code = -1; break; }
    if (cntf > 0 || zg > 0) {
      for (int p = threadIdx.x; p < npx; p += blockDim.x) tmp[p] = tg[p] != 0;
      __syncthreads();
      bwselect_block(tmp, bwg, m, m, c, c, 8);
      int anyzero = 0;
      for (int p = threadIdx.x; p < npx; p += blockDim.x) anyzero |= !bwg[p];
      if (!__syncthreads_or(anyzero)) bwselect_block(mtile, bwg, m, m, c, c, 8);
      int cnt = 0;
      for (int p = threadIdx.x; p < npx; p += blockDim.x) {
        tg[p] *= (double)bwg[p];
        cnt += bwg[p];
      }
      cg = block_sum_int(cnt, sh.ired);
    }
    double meang, bottomg;
    masked_stats(tg, npx, sh.red, &meang, &bottomg);
    double b2[6] = {0, 0, 0, 0, 0, 0};
    for (int p = threadIdx.x; p < npx; p += blockDim.x) {
      const int i = p % m, j = p / m;
      double gx, gy, dx, dy, rfp;
      if (cc.jg) {
        gx = gxs[p]; gy = gys[p]; dx = dxl[i]; dy = dyl[j];
      } else {
        const double s = (double)bwf[p];
        gx = fr.GX(x1 + i, y1 + j) * s; gy = fr.GY(x1 + i, y1 + j) * s;
        dx = (double)(x1 + i - x0); dy = (double)(y1 + j - y0);
      }
      if (cc.rf) {
        rfp = rf[p];
      } else {
        const double fv = fr.F(x1 + i, y1 + j) * fr.M(x1 + i, y1 + j) * (double)bwf[p];
        rfp = (fv - meanf) / bottomf;
      }
      const double r = rfp - (tg[p] - meang) / bottomg;
      b2[0] += dx * gx * r;
      b2[1] += dx * gy * r;
      b2[2] += dy * gx * r;
      b2[3] += dy * gy * r;
      b2[4] += gx * r;
      b2[5] += gy * r;
    }
    block_sum<6>(b2, sh.red);
    // control on thread 0, broadcast through shared memory
    if (threadIdx.x == 0) {
      double b[6], nb = 0;
      for (int k = 0; k < 6; ++k) { b[k] = bottomf * b2[k]; nb += b[k] * b[k]; }
      double nN = sqrt(nb);
      const double nA = nN;
      if (step == 1) sh.red[0] = nN;  // normInit
      const double nI = step == 1 ? nN : normInit;
      if (nI > tol) nN = nN / nI;
      else nN = 0;
      int done = 0;
      if (nN < tol || nA < tol) done = 1;
      else {
        double D[6];
        if (sh.hm_spd) chol6_solve(sh.L, b, D);
        else small_solve(sh.Hm, b, 6, D);
        for (int k = 0; k < 6; ++k) D[k] = -D[k];
        double Pn[6];
        for (int k = 0; k < 6; ++k) Pn[k] = P[k];
        if (!compose_update(Pn, D)) done = 2;
        for (int k = 0; k < 6; ++k) sh.P[k] = Pn[k];
      }
      sh.red[1] = nN;
      sh.red[2] = nA;
      sh.flag = done;
      if (done) for (int k = 0; k < 6; ++k) sh.P[k] = P[k];
    }
    __syncthreads();
    if (step == 1) normInit = sh.red[0];
    normNew = sh.red[1];
    normAbs = sh.red[2];
    const int done = sh.flag;
    for (int k = 0; k < 6; ++k) P[k] = sh.P[k];
    __syncthreads();
    if (done) break;
  }
  if (code == -1) { finish(-1, true, P, nullptr); return; }
  int st = step;
  if (!(normNew < tol || normAbs < tol)) st = kMaxIter + 1;
  if (isnan(normNew)) st = kMaxIter + 1;
  if (sabs < 1e-6) st = kMaxIter + 3;
  finish(st, false, P, sh.Hm);
}

// ---------------------------------------------------------------------------
// 2-DOF augmented-Lagrangian Subpb1 (funICGN_Subpb1.m).  Dynamic shared
// memory as for the 6-DOF kernel plus npx_cap doubles for tempf.
// ---------------------------------------------------------------------------
__device__ void plain2_node(const IcgnArgs& a, const int node, unsigned char* dsm, Shared& sh,
                            const int npx_cap) {
  Frame64 fr{(const double*)a.f, (const double*)a.g, a.mask, (const double*)a.dfdx,
             (const double*)a.dfdy, a.W, a.H};
  double* tg = (double*)dsm;
  double* tf = tg + npx_cap;
  uint8_t* mtile = (uint8_t*)(tf + npx_cap);
  uint8_t* bwf = mtile + npx_cap;
  uint8_t* bwg = bwf + npx_cap;
  uint8_t* tmp = bwg + npx_cap;

  const long long x0 = llround(a.coords[node]), y0 = llround(a.coords[a.N + node]);
  int wx = a.wsl2[node], wy = a.wsl2[a.N + node];
  const double tol = a.tol, mu = a.mu;
  const double UOx = a.UOld[2 * node], UOy = a.UOld[2 * node + 1];
  const double vdx = a.vdual[2 * node], vdy = a.vdual[2 * node + 1];
  double P[6] = {a.FOld[4 * node], a.FOld[4 * node + 1], a.FOld[4 * node + 2],
                 a.FOld[4 * node + 3], UOx, UOy};

  auto finish = [&](int code, bool nan_out) {
    if (threadIdx.x == 0) {
      a.conv[node] = code;
      a.U[2 * node] = nan_out ? nan("") : P[4];
      a.U[2 * node + 1] = nan_out ? nan("") : P[5];
    }
  };
  long long x1 = x0 - wx / 2, x3 = x0 + wx / 2, y1 = y0 - wy / 2, y3 = y0 + wy / 2;
  if ((wx & 1) || (wy & 1) || wx < 0 || wy < 0 || !mask_crop_ok(fr, x1, x3, y1, y3) ||
      !crop_ok(fr, x1, x3, y1, y3) || (wx + 1) * (wy + 1) > npx_cap) {
    finish(0, true);
    return;
  }
  int cntf = 0, nanf = 0;
  {
    const int mx = wx + 1, npx = (wx + 1) * (wy + 1);
    for (int p = threadIdx.x; p < npx; p += blockDim.x) {
      const int i = p % mx, j = p / mx;
      const double t = fr.F(x1 + i, y1 + j) * fr.M(x1 + i, y1 + j);
      if (t != t) nanf = 1;
      if (t == 0) ++cntf;
    }
  }
  cntf = block_sum_int(cntf, sh.ired);
  if (__syncthreads_or(nanf)) { finish(0, true); return; }
  const double npx0 = (double)(wx + 1) * (double)(wy + 1);
  if (!((double)cntf < 0.4 * npx0)) { finish(kMaxIter + 2, false); return; }
  if ((double)cntf > 0.0 * npx0) {
    {
      const double aa = (double)(wx + 1) * (double)(wy + 1);
      wx = (int)grow_window(aa, aa - (double)cntf, wx);
    }
    {
      const double aa = (double)(wx + 1) * (double)(wy + 1);
      wy = (int)grow_window(aa, aa - (double)cntf, wy);
    }
    x1 = x0 - wx / 2; x3 = x0 + wx / 2; y1 = y0 - wy / 2; y3 = y0 + wy / 2;
    if (!mask_crop_ok(fr, x1, x3, y1, y3) || !crop_ok(fr, x1, x3, y1, y3) ||
        (wx + 1) * (wy + 1) > npx_cap) {
      finish(0, true);
      return;
    }
  }
  const int mx = wx + 1, my = wy + 1, npx = mx * my;
  const int sc = (wx + 1) / 2, sr = (wy + 1) / 2;  // bwselect(BW, c, r): column, row
  bool has_masked;
  {
    int z = 0;
    for (int p = threadIdx.x; p < npx; p += blockDim.x) {
      const int i = p % mx, j = p / mx;
      const uint8_t mk = __ldg(fr.mask + (y1 + j - 1) * fr.W + (x1 + i - 1)) != 0;
      mtile[p] = mk;
      if (!mk) z = 1;
    }
    has_masked = __syncthreads_or(z) != 0;
  }
  if (has_masked) bwselect_block(mtile, bwf, mx, my, sr, sc, 4);
  else {
    for (int p = threadIdx.x; p < npx; p += blockDim.x) bwf[p] = 1;
    __syncthreads();
  }
  // bw points at the selection that currently masks tempf/DfDx/DfDy
  const uint8_t* bw = bwf;
  auto f_stats = [&](double* A11, double* A12, double* A22, double* mf, double* bf) {
    double h[3] = {0, 0, 0};
    for (int p = threadIdx.x; p < npx; p += blockDim.x) {
      const int i = p % mx, j = p / mx;
      const double s = (double)bw[p];
      const double gx = fr.GX(x1 + i, y1 + j) * s, gy = fr.GY(x1 + i, y1 + j) * s;
      tf[p] = fr.F(x1 + i, y1 + j) * fr.M(x1 + i, y1 + j) * s;
      h[0] += gx * gx; h[1] += gx * gy; h[2] += gy * gy;
    }
    block_sum<3>(h, sh.red);
    masked_stats(tf, npx, sh.red, mf, bf);
    const double b2 = *bf * *bf;
    *A11 = h[0] * 2 / b2 + mu;
    *A12 = h[1] * 2 / b2;
    *A22 = h[2] * 2 / b2 + mu;
  };
  double A11, A12, A22, meanf, bottomf;
  f_stats(&A11, &A12, &A22, &meanf, &bottomf);

  double normNew = 1, normAbs = 1, normInit = 0;
  int step = 0;
  while (step <= 100 && normNew > tol && normAbs > tol) {
    ++step;
    if (any_oob(fr, P, x0, y0, x1, y1, mx, my)) { normNew = 1e6; break; }
    int zg = 0, nang = 0;
    for (int p = threadIdx.x; p < npx; p += blockDim.x) {
      const int i = p % mx, j = p / mx;
      double u22, v22;
      warp_exact(P, (double)(x1 + i - x0), (double)(y1 + j - y0), (double)x0, (double)y0, &u22, &v22);
      const double t = ba_cubic_exact(fr.g, fr.W, fr.H, v22, u22);
      tg[p] = t;
      if (t != t) nang = 1;
      if (t == 0) ++zg;
    }
    zg = block_sum_int(zg, sh.ired);
    if (__syncthreads_or(nang)) { step = -1; break; }
    if (cntf > 0 || zg > 0) {
      for (int p = threadIdx.x; p < npx; p += blockDim.x) tmp[p] = tg[p] != 0;
      __syncthreads();
      bwselect_block(tmp, bwg, mx, my, sr, sc, 4);
      int anyzero = 0;
      for (int p = threadIdx.x; p < npx; p += blockDim.x) anyzero |= !bwg[p];
      if (!__syncthreads_or(anyzero)) bwselect_block(mtile, bwg, mx, my, sr, sc, 8);
      for (int p = threadIdx.x; p < npx; p += blockDim.x) tg[p] *= (double)bwg[p];
      __syncthreads();
      bw = bwg;  // tempf, DfDx, DfDy, H, meanf, bottomf recomputed with tempg_BW2
      f_stats(&A11, &A12, &A22, &meanf, &bottomf);
    }
    double meang, bottomg;
    masked_stats(tg, npx, sh.red, &meang, &bottomg);
    double b2[2] = {0, 0};
    for (int p = threadIdx.x; p < npx; p += blockDim.x) {
      const int i = p % mx, j = p / mx;
      const double s = (double)bw[p];
      const double gx = fr.GX(x1 + i, y1 + j) * s, gy = fr.GY(x1 + i, y1 + j) * s;
      const double r = (tf[p] - meanf) / bottomf - (tg[p] - meang) / bottomg;
      b2[0] += gx * r;
      b2[1] += gy * r;
    }
    block_sum<2>(b2, sh.red);
    if (threadIdx.x == 0) {
      const double b0 = bottomf * b2[0], b1 = bottomf * b2[1];
      const double tb0 = b0 * 2 / (bottomf * bottomf) + mu * (P[4] - UOx - vdx);
      const double tb1 = b1 * 2 / (bottomf * bottomf) + mu * (P[5] - UOy - vdy);
      const double dmax = isnan(A11) ? A22 : (isnan(A22) ? A11 : fmax(A11, A22));
      const double Hm[4] = {A11 + 1e-3 * dmax, A12, A12, A22 + 1e-3 * dmax};
      const double rhs[2] = {tb0, tb1};
      double dP[2];
      small_solve(Hm, rhs, 2, dP);
      double nN = sqrt(tb0 * tb0 + tb1 * tb1);
      const double nA = nN;
      const double nI = step == 1 ? nN : normInit;
      if (step == 1) sh.red[0] = nN;
      if (nI > tol) nN = nN / nI;
      else nN = 0;
      int done = 0;
      double Pn[6];
      for (int k = 0; k < 6; ++k) Pn[k] = P[k];
      if (nN < tol || nA < tol) done = 1;
      else {
        const double D[6] = {0, 0, 0, 0, -dP[0], -dP[1]};
        if (!compose_update(Pn, D)) done = 2;
      }
      for (int k = 0; k < 6; ++k) sh.P[k] = Pn[k];
      sh.red[1] = nN;
      sh.red[2] = nA;
      sh.flag = done;
    }
    __syncthreads();
    if (step == 1) normInit = sh.red[0];
    normNew = sh.red[1];
    normAbs = sh.red[2];
    const int done = sh.flag;
    for (int k = 0; k < 6; ++k) P[k] = sh.P[k];
    __syncthreads();
    if (done) break;
  }
  if (step == -1) { finish(0, true); return; }
  int st = step;
  if (!(normNew < tol || normAbs < tol)) st = kMaxIter + 1;
  if (isnan(normNew)) st = kMaxIter + 1;
  double v[1] = {0};
  for (int p = threadIdx.x; p < npx; p += blockDim.x) v[0] += fabs(tf[p]);
  block_sum<1>(v, sh.red);
  if (v[0] < 1e-6) st = kMaxIter + 3;
  finish(st, false);
}

// ---------------------------------------------------------------------------
// Size classes.  Every node runs on one CTA, as in the reference's per-node
// loop; the nodes are sorted by subset size and each class runs with a CTA
// sized to its tiles (fewer idle threads, and shared memory for its own grown
// tile instead of the largest one of the call), so that many more small
// subsets are in flight on an SM.  Persistent CTAs stride over their class.
// ---------------------------------------------------------------------------
namespace {

struct PlainClass {
  const int32_t* order;  // node order (sorted by size); nullptr: nodes 0..N-1
  const int* range;      // [lo, hi) of this class in order; nullptr: [0, N)
  int npx_cap;           // tile capacity of the CTA's shared memory
  int* head;             // work counter of the class (zero at launch)
  PlainCache cache;      // 6-DOF: per-pixel terms kept in shared memory
};

template <int T, bool TWO>
__global__ void __launch_bounds__(T) icgn_plain_class_kernel(IcgnArgs a, PlainClass cl) {
  extern __shared__ __align__(16) unsigned char dsm[];
  __shared__ Shared sh;
  const int lo = cl.range ? cl.range[0] : 0, hi = cl.range ? cl.range[1] : a.N;
  // CTAs pull nodes from the class's counter: iteration counts vary by two
  // orders of magnitude, and a fixed stride left some SMs working twice as
  // long as the mean
  __shared__ int s_q;
  for (;;) {
    if (threadIdx.x == 0) s_q = lo + atomicAdd(cl.head, 1);
    __syncthreads();
    const int q = s_q;
    if (q >= hi) break;
    const int node = cl.order ? cl.order[q] : q;
    if constexpr (TWO) plain2_node(a, node, dsm, sh, cl.npx_cap);
    else plain6_node(a, node, dsm, sh, cl.npx_cap, cl.cache);
    __syncthreads();  // thread 0's output writes read sh before the next node reuses it
  }
}

// Class k covers subset edges (kClassEdge[k-1], kClassEdge[k]]; the last class
// takes everything larger.
constexpr int kClasses = 4;
constexpr int kClassEdge[kClasses] = {8, 16, 32, 255};
constexpr int kClassThreads[kClasses] = {32, 64, 128, 256};

// Queue positions of each class from the histogram of subset edges of an
// ascending queue (bin b = edge b).
__global__ void plain_class_ranges_kernel(const int* __restrict__ hist, int* ranges, int4 edges) {
  if (threadIdx.x != 0) return;
  const int e[kClasses] = {edges.x, edges.y, edges.z, edges.w};
  int pos = 0, b = 0;
  for (int k = 0; k < kClasses; ++k) {
    ranges[2 * kClasses + k] = 0;  // the class's work counter
    ranges[2 * k] = pos;
    for (; b <= e[k]; ++b) pos += hist[b];
    ranges[2 * k + 1] = pos;
  }
}

template <int T, bool TWO>
cudaError_t launch_class(const IcgnArgs& a, PlainClass cl, int nodes_hint, cudaStream_t s) {
  size_t smem;
  if (TWO) {
    cl.cache = PlainCache{0, 0};
    smem = (size_t)cl.npx_cap * (2 * sizeof(double) + 4);
  } else {
    // the 6-DOF kernel keeps as many of its fixed per-pixel terms in shared
    // memory as 200 KB of it allows (every class but the largest tiles'
    // keeps both; the occupancy of these classes is set by registers)
    constexpr size_t kLimit = 200 * 1024;
    cl.cache = PlainCache{1, 1};
    if (plain6_smem_bytes(cl.npx_cap, cl.cache) > kLimit) cl.cache.jg = 0;
    if (plain6_smem_bytes(cl.npx_cap, cl.cache) > kLimit) cl.cache.rf = 0;
    smem = plain6_smem_bytes(cl.npx_cap, cl.cache);
  }
  cudaError_t e = cudaFuncSetAttribute(icgn_plain_class_kernel<T, TWO>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  // resident CTAs per SM for this shared-memory size, queried once (the
  // first call of a loop runs before any graph capture of it)
  static int cached_smem[64] = {}, cached_per_sm[64] = {};
  int per_sm = 0;
  for (int k = 0; k < 64 && cached_smem[k]; ++k)
    if (cached_smem[k] == (int)smem) { per_sm = cached_per_sm[k]; break; }
  if (per_sm == 0) {
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, icgn_plain_class_kernel<T, TWO>, T, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    for (int k = 0; k < 64; ++k)
      if (!cached_smem[k]) { cached_smem[k] = (int)smem; cached_per_sm[k] = per_sm; break; }
  }
  int blocks = current_sm_count() * per_sm;
  if (nodes_hint > 0 && nodes_hint < blocks) blocks = nodes_hint;
  icgn_plain_class_kernel<T, TWO><<<blocks, T, smem, s>>>(a, cl);
  return cudaGetLastError();
}

template <bool TWO>
cudaError_t launch_plain(const IcgnArgs& a, int32_t* order, int* qscratch, int* ranges, cudaStream_t s,
                         int* kernels, const PlainStreams* ps) {
  *kernels = 0;
  if (a.N <= 0) return cudaSuccess;
  const bool per_node = TWO ? a.wsl2 != nullptr : a.ws_list != nullptr;
  if (!per_node) {
    // one subset size: one class
    const int ws = a.ws_all;
    PlainClass cl{nullptr, nullptr, a.npx_max, ranges + 2 * kClasses};
    cudaError_t e = cudaMemsetAsync(cl.head, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    *kernels = 1;
    if (ws <= 8) return launch_class<32, TWO>(a, cl, a.N, s);
    if (ws <= 16) return launch_class<64, TWO>(a, cl, a.N, s);
    if (ws <= 32) return launch_class<128, TWO>(a, cl, a.N, s);
    return launch_class<256, TWO>(a, cl, a.N, s);
  }
  cudaError_t e = launch_build_queue(TWO ? nullptr : a.ws_list, TWO ? a.wsl2 : nullptr, a.ws_all, a.N, order,
                                     nullptr, qscratch, s, 1, 0);
  if (e != cudaSuccess) return e;
  plain_class_ranges_kernel<<<1, 32, 0, s>>>(
      qscratch, ranges, make_int4(kClassEdge[0], kClassEdge[1], kClassEdge[2], kClassEdge[3]));
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  *kernels = 4;
  // The classes run concurrently when side streams are given: each class is
  // a persistent grid that fills the SMs, so a later class's CTAs start as
  // the earlier class drains, and the slow subsets at the end of one class
  // (3 to 101 iterations each) overlap the next class's work instead of
  // leaving SMs idle.  The 8-px class, whose long subsets make the longest
  // tail, is launched first.
  if (ps) {
    e = cudaEventRecord(ps->fork, s);
    if (e != cudaSuccess) return e;
  }
  int forked = 0;
  for (int k = 0; k < kClasses && e == cudaSuccess; ++k) {
    PlainClass cl{order, ranges + 2 * k, k + 1 < kClasses ? std::min(grown_tile_pixels(kClassEdge[k]), a.npx_max)
                                                           : a.npx_max,
                  ranges + 2 * kClasses + k};
    cudaStream_t sk = s;
    if (ps && k > 0) {
      sk = ps->side[k - 1];
      e = cudaStreamWaitEvent(sk, ps->fork, 0);
      if (e != cudaSuccess) break;
    }
    switch (kClassThreads[k]) {
      case 32: e = launch_class<32, TWO>(a, cl, a.N, sk); break;
      case 64: e = launch_class<64, TWO>(a, cl, a.N, sk); break;
      case 128: e = launch_class<128, TWO>(a, cl, a.N, sk); break;
      default: e = launch_class<256, TWO>(a, cl, a.N, sk); break;
    }
    if (ps && k > 0) {
      const cudaError_t e2 = cudaEventRecord(ps->join[k - 1], sk);
      if (e == cudaSuccess) e = e2;
      if (e2 == cudaSuccess) ++forked;
    }
    ++*kernels;
  }
  // every side stream that was given work is joined back, errors or not
  for (int k = 0; k < forked; ++k) {
    const cudaError_t e2 = cudaStreamWaitEvent(s, ps->join[k], 0);
    if (e == cudaSuccess) e = e2;
  }
  return e;
}

}  // namespace

cudaError_t launch_icgn6_plain(const IcgnArgs& a, int32_t* order, int* qscratch, int* ranges, cudaStream_t s,
                               int* kernels, const PlainStreams* ps) {
  return launch_plain<false>(a, order, qscratch, ranges, s, kernels, ps);
}

cudaError_t launch_icgn2_plain(const IcgnArgs& a, int32_t* order, int* qscratch, int* ranges, cudaStream_t s,
                               int* kernels, const PlainStreams* ps) {
  return launch_plain<true>(a, order, qscratch, ranges, s, kernels, ps);
}

}  // namespace stdic
