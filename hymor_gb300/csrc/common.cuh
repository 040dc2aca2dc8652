// Shared device-side definitions of libhymor (sm_103a).
//
// Layout in HBM (all FP64, column-major, chi index fastest, like the reference):
//   ghosted cell arrays  G = (Nchi+2) x (Neta+2)   conserved variables, p, T, a
//   cell arrays          N = Nchi x Neta            fluxes, 1/volume
//   lr faces             (Nchi+1) x Neta            6 SoA geometry planes
//   bt faces             Nchi x (Neta+1)            6 SoA geometry planes
// Every array is a separate cudaMalloc (256-byte aligned base), SoA by variable.
#pragma once

#include <cstdint>
#include <cuda.h>  // CUtensorMap (the TMA descriptors of the flux halo)
#include <cuda_runtime.h>

#include "../../include/hymor.h"

namespace hymor {

constexpr int kWarp = 32;

// Face geometry planes (precomputed once per mesh, hymor_ctx_create), with s = 2 / Re:
//   lr face (i, j), between ghosted cells (i, j+1) and (i+1, j+1):
//     0 nx, 1 ny, 2 A/2, 3 s g1 = -s / (cld * Cn1_Fn1), 4 s g2/4 = -s Cn1_Ft1 / (4 len Cn1_Fn1), 5 s/(4 len)
//   bt face (i, j), between ghosted cells (i+1, j) and (i+1, j+1):
//     0 nx, 1 ny, 2 A/2, 3 s h1 = s / (cbd * Cn2_Fn2),  4 s h2/4 = s Cn2_Ft2 / (4 len Cn2_Fn2),   5 s/(4 len)
// so that, with U_c = 4 u_c the sum of the four cells around a corner, the gradients of
// VISCOUS_FLUX.jl:98-127 come out multiplied by s:
//   s du_dn1 = (s g1) (u_R - u_L) + (s g2/4) (U_c(i, j+1) - U_c(i, j)),  s du_dt1 =  (s/(4 len)) (U_c(i,j+1) - U_c(i,j))
//   s du_dn2 = (s h1) (u_T - u_B) + (s h2/4) (U_c(i+1, j) - U_c(i, j)),  s du_dt2 = -(s/(4 len)) (U_c(i+1,j) - U_c(i,j))
// and the traction formed from them is twice mu/Re times the unit-viscosity traction.
constexpr int kGeoPlanes = 6;

struct DevMesh {
  int nchi, neta;
  const double *lr_xn, *lr_yn, *lr_a, *bt_xn, *bt_yn, *bt_a, *vol;
  const double *x_ext, *y_ext, *x_corner, *y_corner, *chi1, *fb_area;
  double fb_yn_front, fb_yn_back;
  const double* lrg;   // kGeoPlanes x NLR
  const double* btg;   // kGeoPlanes x NBT
  const double* rvol;  // N
  const double* rx_lr;  // axisymmetric: (2 / Re) / x_face on lr faces (NLR)
  const double* rx_bt;  // axisymmetric: (2 / Re) / x_face on bt faces (NBT)
  const double* gvis;   // kv 2 (A_xi^2 + A_eta^2) / vol^2 per cell, kv = max(4/3, gamma/Pr) / Re
                        // (viscous CFL rate over the volume, CFL_TIMESTEP.jl:110-113)
  const double *xt, *yt;  // x_ext, y_ext transposed: ghosted (i, j) at i * (Neta + 2) + j
  // float-float copies (high, low) of the lr / bt face planes nx, ny, s g1 (s h1), s g2/4
  // (s h2/4), s/(4 len), A/2, 6 x NLR and 6 x NBT, for the float-float viscous terms of the
  // RK-step flux
  const float2* lrf;
  const float2* btf;
  // nx A/2, ny A/2 (FP64, 2 x NLR and 2 x NBT): the inviscid face fluxes of the RK step with
  // the area folded into the normal
  const double* lra;
  const double* bta;
};

struct Cons {
  double *rho, *ru, *rv, *rE;
};

struct ShockPts {
  double *x, *y, *chi, *eta;
};

// Device scalars (one cudaMalloc'd block):
enum Scalar {
  kDt = 0,
  kT = 1,
  kCmax = 2,      // max |a| (bits, non-negative double ordered as uint64)
  kMaxLam = 3,    // max lam_over_V
  kMaxFlux = 4,   // max of the three dt2 terms
  kCount
};

// Error word bits and counters (uint32 block).
enum ErrWord {
  kErrFlags = 0,
  kRhoLimited = 1,
  kRhWarn = 2,
  kErrCount
};
enum ErrBit : unsigned {
  kBitNumeric = 1u,
  kBitShockRange = 2u,
  kBitTimeout = 4u,  // a bounded wait on a TMA transfer gave up
};

// TMA descriptors of the six halo planes a flux launch reads (rho, rho_u, rho_v, rho_E, p, T
// of the array evaluated), passed by value as a __grid_constant__ kernel parameter.
struct FluxMaps {
  CUtensorMap m[6];
};

__host__ __device__ inline int gidx(int i, int j, int nchi) { return i + j * (nchi + 2); }  // 0-based ghosted

// Reciprocal by the hardware seed (rcp.approx.ftz.f64, ~20 correct bits) refined
// with one cubic Newton–Raphson (Householder order-3) step: e = 1 - x r,
// r' = r (1 + e + e^2); relative error ~ e^3 < 2^-60 before rounding, i.e. within
// about 1 ulp of 1/x. Three DFMA instead of the ~10-DFMA-equivalent IEEE divide.
__device__ __forceinline__ double frcp(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  double e = fma(-x, r, 1.0);
  double e2 = fma(e, e, e);
  return fma(r, e2, r);
}

__device__ __forceinline__ double jsign(double x) { return x > 0 ? 1.0 : (x < 0 ? -1.0 : x); }

// max over non-negative doubles through their ordered bit patterns
__device__ __forceinline__ void atomic_max_nonneg(double* addr, double v) {
  if (!(v >= 0)) v = (v != v) ? __longlong_as_double(0x7ff0000000000000LL) : 0.0;  // NaN -> +inf
  atomicMax(reinterpret_cast<unsigned long long*>(addr), (unsigned long long)__double_as_longlong(v));
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

}  // namespace hymor
