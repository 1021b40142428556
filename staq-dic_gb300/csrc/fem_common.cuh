// Q4 shape functions with the four optional hanging (mid-edge) nodes and the
// Gauss rules of the reference's quadtree FEM (func_quadtree/Subpb2Quadtree.m
// and funGlobalNodalStrainQuadtree.m: N1..N8, their ksi/eta derivatives and the
// GaussPtOrder 2..5 points and weights).
#pragma once
#include "device_common.cuh"

namespace stdic {

STDIC_DEV double sgnd(double x) { return (double)((x > 0) - (x < 0)); }

STDIC_DEV void shape(double ksi, double eta, const double dp[4], double Nv[8], double dk[8],
                     double de[8]) {
  const double N5 = dp[0] * 0.5 * (1 + ksi) * (1 - fabs(eta));
  const double N6 = dp[1] * 0.5 * (1 + eta) * (1 - fabs(ksi));
  const double N7 = dp[2] * 0.5 * (1 - ksi) * (1 - fabs(eta));
  const double N8 = dp[3] * 0.5 * (1 - eta) * (1 - fabs(ksi));
  Nv[0] = (1 - ksi) * (1 - eta) * 0.25 - 0.5 * (N7 + N8);
  Nv[1] = (1 + ksi) * (1 - eta) * 0.25 - 0.5 * (N8 + N5);
  Nv[2] = (1 + ksi) * (1 + eta) * 0.25 - 0.5 * (N5 + N6);
  Nv[3] = (1 - ksi) * (1 + eta) * 0.25 - 0.5 * (N6 + N7);
  Nv[4] = N5; Nv[5] = N6; Nv[6] = N7; Nv[7] = N8;
  const double N5k = dp[0] * 0.5 * (1 - fabs(eta)), N5e = dp[0] * 0.5 * (1 + ksi) * sgnd(-eta);
  const double N6k = dp[1] * 0.5 * (1 + eta) * sgnd(-ksi), N6e = dp[1] * 0.5 * (1 - fabs(ksi));
  const double N7k = dp[2] * 0.5 * (-1) * (1 - fabs(eta)), N7e = dp[2] * 0.5 * (1 - ksi) * sgnd(-eta);
  const double N8k = dp[3] * 0.5 * (1 - eta) * sgnd(-ksi), N8e = dp[3] * 0.5 * (-1) * (1 - fabs(ksi));
  dk[0] = -0.25 * (1 - eta) - 0.5 * (N7k + N8k);
  de[0] = -0.25 * (1 - ksi) - 0.5 * (N7e + N8e);
  dk[1] = 0.25 * (1 - eta) - 0.5 * (N8k + N5k);
  de[1] = -0.25 * (1 + ksi) - 0.5 * (N8e + N5e);
  dk[2] = 0.25 * (1 + eta) - 0.5 * (N5k + N6k);
  de[2] = 0.25 * (1 + ksi) - 0.5 * (N5e + N6e);
  dk[3] = -0.25 * (1 + eta) - 0.5 * (N6k + N7k);
  de[3] = 0.25 * (1 - ksi) - 0.5 * (N6e + N7e);
  dk[4] = N5k; de[4] = N5e;
  dk[5] = N6k; de[5] = N6e;
  dk[6] = N7k; de[6] = N7e;
  dk[7] = N8k; de[7] = N8e;
}

STDIC_DEV int gauss_rule(int order, double* pt, double* wt) {
  switch (order) {
    case 2: pt[0] = -1 / sqrt(3.0); pt[1] = 1 / sqrt(3.0); wt[0] = wt[1] = 1; return 2;
    case 3:
      pt[0] = 0; pt[1] = sqrt(3.0 / 5); pt[2] = -sqrt(3.0 / 5);
      wt[0] = 8.0 / 9; wt[1] = 5.0 / 9; wt[2] = 5.0 / 9; return 3;
    case 4:
      pt[0] = 0.339981; pt[1] = -0.339981; pt[2] = 0.861136; pt[3] = -0.861136;
      wt[0] = 0.652145; wt[1] = 0.652145; wt[2] = 0.347855; wt[3] = 0.347855; return 4;
    case 5:
      pt[0] = 0; pt[1] = 0.538469; pt[2] = -0.538469; pt[3] = 0.90618; pt[4] = -0.90618;
      wt[0] = 0.568889; wt[1] = 0.478629; wt[2] = 0.478629; wt[3] = 0.236927; wt[4] = 0.236927;
      return 5;
  }
  return 0;
}


}  // namespace stdic
