// Manufactured-solution sources shared by the RieCG and KozCG kernels.
#pragma once

#include "xg.h"

namespace xg {

// A problem (enum xg_source) with its control-file parameters (alpha,
// beta[3], kappa, r0, p0, ce) and the ratio of specific heats.
struct SrcPrm {
  int problem;
  double p[8];
  double gamma;
};

// Manufactured source s(x, y, z, t) of a problem (riemann::src,
// src/Physics/Riemann.cpp:880-907, with the problems' src functions of
// src/Physics/Problems.cpp: nonlinear_energy_growth 163-220, rayleigh_taylor
// 261-332, taylor_green 433-449, vortical_flow 481-508), in FP64.
__device__ inline void problem_source(const SrcPrm& q, double x, double y, double z, double t,
                                      double o[5]) {
  const double pi = 3.14159265358979323846, g = q.gamma;
  const double a = q.p[0], b0 = q.p[1], b1 = q.p[2], b2 = q.p[3];
  const double kap = q.p[4], r0 = q.p[5], p0 = q.p[6], ce = q.p[7];
#pragma unroll
  for (int c = 0; c < 5; ++c) o[c] = 0.0;
  if (q.problem == XG_SRC_TAYLOR_GREEN) {
    // energy only: 3 pi/8 (cos 3 pi x cos pi y - cos 3 pi y cos pi x)
    o[4] = 3.0 * pi / 8.0 * (cos(3.0 * pi * x) * cos(pi * y) - cos(3.0 * pi * y) * cos(pi * x));
  } else if (q.problem == XG_SRC_VORTICAL_FLOW) {
    // unit density, momentum (a x - k y, k x + a y, -2 a z)
    const double rho = 1.0, mx = a * x - kap * y, my = kap * x + a * y;
    o[1] = a * mx / rho - kap * my / rho;
    o[2] = kap * mx / rho + a * my / rho;
    o[4] = (o[1] * mx + o[2] * my) / rho + 8.0 * a * a * a * z * z / (g - 1.0);
  } else if (q.problem == XG_SRC_NONLINEAR_ENERGY_GROWTH) {
    // rho = r0 + exp(-a t)(1 - |x|^2), e = (-3 (ce + k h^2 t))^(-1/3),
    // h = cos(b0 pi x) cos(b1 pi y) cos(b2 pi z)
    const double gx = 1.0 - x * x - y * y - z * z;
    const double dg[3] = {-2.0 * x, -2.0 * y, -2.0 * z};
    const double cx = cos(b0 * pi * x), cy = cos(b1 * pi * y), cz = cos(b2 * pi * z);
    const double h = cx * cy * cz;
    const double dh[3] = {-b0 * pi * sin(b0 * pi * x) * cy * cz, -b1 * pi * cx * sin(b1 * pi * y) * cz,
                          -b2 * pi * cx * cy * sin(b2 * pi * z)};
    const double ft = exp(-a * t), dfdt = -a * ft;
    const double rho = r0 + ft * gx, drdt = gx * dfdt;
    const double ie = pow(-3.0 * (ce + kap * h * h * t), -1.0 / 3.0);
    const double ie4 = pow(ie, 4.0);
    o[0] = drdt;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const double dedx = 2.0 * ie4 * kap * h * dh[j] * t, drdx = ft * dg[j];
      o[1 + j] = (g - 1.0) * (rho * dedx + ie * drdx);
    }
    o[4] = rho * (kap * h * h * ie4) + ie * drdt;
  } else if (q.problem == XG_SRC_RAYLEIGH_TAYLOR) {
    // rho = r0 - |b x^2|, p = p0 + a |b x^2|, velocity cos(k pi t) times
    // (z sin pi x, z cos pi y, -pi z^2 (cos pi x - sin pi y) / 2); the
    // conserved solution formed first and the primitives taken from it
    const double gx = b0 * x * x + b1 * y * y + b2 * z * z;
    const double ft = cos(kap * pi * t), st = sin(kap * pi * t);
    const double sx = sin(pi * x), cx = cos(pi * x), sy = sin(pi * y), cy = cos(pi * y);
    const double r = r0 - gx;
    const double u0 = ft * z * sx, v0 = ft * z * cy, w0 = ft * (-0.5 * pi * z * z * (cx - sy));
    const double rE = (p0 + a * gx) / (g - 1.0) + 0.5 * r * (u0 * u0 + v0 * v0 + w0 * w0);
    const double m[3] = {r * u0, r * v0, r * w0};
    const double rho = r, u = m[0] / rho, v = m[1] / rho, w = m[2] / rho, E = rE / rho;
    const double p = p0 + a * (b0 * x * x + b1 * y * y + b2 * z * z);
    const double drdx[3] = {-2.0 * b0 * x, -2.0 * b1 * y, -2.0 * b2 * z};
    const double dpdx[3] = {2.0 * a * b0 * x, 2.0 * a * b1 * y, 2.0 * a * b2 * z};
    const double dudx[3] = {ft * pi * z * cx, 0.0, ft * sx};
    const double dvdx[3] = {0.0, -ft * pi * z * sy, ft * cy};
    const double dwdx[3] = {ft * pi * 0.5 * pi * z * z * sx, ft * pi * 0.5 * pi * z * z * cy,
                            -ft * pi * z * (cx - sy)};
    double dedx[3];
#pragma unroll
    for (int j = 0; j < 3; ++j)
      dedx[j] = dpdx[j] / rho / (g - 1.0) - p / (g - 1.0) / rho / rho * drdx[j] + u * dudx[j] +
                v * dvdx[j] + w * dwdx[j];
    const double dudt = -kap * pi * st * z * sx, dvdt = -kap * pi * st * z * cy;
    const double dwdt = kap * pi * st / 2.0 * pi * z * z * (cx - sy);
    const double dedt = u * dudt + v * dvdt + w * dwdt;
    o[0] = u * drdx[0] + v * drdx[1] + w * drdx[2];
    o[1] = rho * dudt + u * o[0] + dpdx[0] + m[0] * dudx[0] + m[1] * dudx[1] + m[2] * dudx[2];
    o[2] = rho * dvdt + v * o[0] + dpdx[1] + m[0] * dvdx[0] + m[1] * dvdx[1] + m[2] * dvdx[2];
    o[3] = rho * dwdt + w * o[0] + dpdx[2] + m[0] * dwdx[0] + m[1] * dwdx[1] + m[2] * dwdx[2];
    o[4] = rho * dedt + E * o[0] + m[0] * dedx[0] + m[1] * dedx[1] + m[2] * dedx[2] +
           u * dpdx[0] + v * dpdx[1] + w * dpdx[2];
  }
}


// The problems' analytic states at (x, y, z, t), conserved variables (the
// problems' ic functions, src/Physics/Problems.cpp: nonlinear_energy_growth
// 117-151, rayleigh_taylor 226-258, taylor_green 409-428, vortical_flow
// 453-478, total energy as eos::totalenergy, src/Physics/EOS.hpp:53-56).
__device__ inline void problem_ic(const SrcPrm& q, double x, double y, double z, double t,
                                  double o[5]) {
  const double pi = 3.14159265358979323846, g = q.gamma;
  const double a = q.p[0], b0 = q.p[1], b1 = q.p[2], b2 = q.p[3];
  const double kap = q.p[4], r0 = q.p[5], p0 = q.p[6], ce = q.p[7];
  if (q.problem == XG_SRC_TAYLOR_GREEN) {
    const double r = 1.0;
    const double p = 10.0 + r / 4.0 * (cos(2.0 * pi * x) + cos(2.0 * pi * y));
    const double u = sin(pi * x) * cos(pi * y), v = -cos(pi * x) * sin(pi * y), w = 0.0;
    o[0] = r;
    o[1] = r * u;
    o[2] = r * v;
    o[3] = r * w;
    o[4] = p / (g - 1.0) + 0.5 * r * (u * u + v * v + w * w);
  } else if (q.problem == XG_SRC_VORTICAL_FLOW) {
    const double ru = a * x - kap * y, rv = kap * x + a * y, rw = -2.0 * a * z;
    o[0] = 1.0;
    o[1] = ru;
    o[2] = rv;
    o[3] = rw;
    o[4] = (ru * ru + rv * rv + rw * rw) / 2.0 + (p0 - 2.0 * a * a * z * z) / (g - 1.0);
  } else if (q.problem == XG_SRC_NONLINEAR_ENERGY_GROWTH) {
    const double h = cos(b0 * pi * x) * cos(b1 * pi * y) * cos(b2 * pi * z);
    const double r = r0 + exp(-a * t) * (1.0 - x * x - y * y - z * z);
    o[0] = r;
    o[1] = 0.0;
    o[2] = 0.0;
    o[3] = 0.0;
    o[4] = r * pow(-3.0 * (ce + kap * h * h * t), -1.0 / 3.0);
  } else {  // rayleigh_taylor
    const double gx = b0 * x * x + b1 * y * y + b2 * z * z;
    const double r = r0 - gx;
    const double ft = cos(kap * pi * t);
    const double u = ft * z * sin(pi * x), v = ft * z * cos(pi * y);
    const double w = ft * (-0.5 * pi * z * z * (cos(pi * x) - sin(pi * y)));
    o[0] = r;
    o[1] = r * u;
    o[2] = r * v;
    o[3] = r * w;
    o[4] = (p0 + a * gx) / (g - 1.0) + 0.5 * r * (u * u + v * v + w * w);
  }
}

// Dirichlet values of a node at time t (physics::dirbc, src/Physics/
// BC.cpp:30-71): with a problem set, components of mask 1 take its analytic
// state at t; any other set component its given value.
__device__ inline void dirichlet(const SrcPrm& q, double x, double y, double z, double t,
                                 const int32_t* mask, const double* val, double u[5]) {
  double ic[5];
  const bool prob = q.problem != XG_SRC_NONE;
  if (prob) problem_ic(q, x, y, z, t, ic);
#pragma unroll
  for (int c = 0; c < 5; ++c) {
    if (mask[c] == 1 && prob)
      u[c] = ic[c];
    else if (mask[c])
      u[c] = val[c];
  }
}

}  // namespace xg
