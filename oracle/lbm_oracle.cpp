// CPU restatement of taichi-lbm's per-step D2Q9 path: the parity ORACLE.
//
// Test infrastructure only.  Nothing in the product links, loads or calls
// this file; the tests, the smoke check and the benchmark's CPU-baseline leg
// use it as the checker.
//
// Each function restates one reference Taichi kernel, kernel for kernel and
// in the reference's call order, with the reference's field layout
// (node (i, j) at i*NY + j, populations innermost) and with every arithmetic
// expression evaluated in the same order as the reference source, so that
// with -ffp-contract=off the float build reproduces an IEEE serial execution
// of the reference bit for bit (libm exp/pow aside).  Templated on float and
// double (the reference's default_fp f32 / f64).
//
// Parity pin: checked against fixtures produced by running the reference's
// own taichi_lbm source under a serial Taichi stand-in (tests/golden/).
//
// Reference files (paths inside the taichi-lbm project):
//   taichi_lbm/lbm.py                 LBField, MacroscopicEngine
//   taichi_lbm/CollisionEngine.py     Collision, BGK/TRT/MRT
//   taichi_lbm/FluidModels.py         Newtonian, power law
//   taichi_lbm/EOS.py                 pseudopotentials
//   taichi_lbm/ExternalForce.py       ShanChenForceC1
//   taichi_lbm/SCBoundaryCondition.py psi boundaries
//   taichi_lbm/BoundaryCondition.py   grouping, stream carriers, BCs
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

namespace {

// lbm.py:44-45 — D2Q9 velocity set and weights, in the reference's order
const int CX[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
const int CY[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
// BoundaryCondition.py:242 — bounce map
const int OPP[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};

// BoundaryCondition.py:63-72 — PlaneBoundary unknown populations per direction
void unknowns(int dir, int out[3]) {
  static const int U1[3] = {3, 6, 7}, U3[3] = {1, 5, 8}, U4[3] = {2, 5, 6}, U2[3] = {4, 7, 8};
  const int* u = dir == 1 ? U1 : dir == 3 ? U3 : dir == 4 ? U4 : U2;
  for (int k = 0; k < 3; ++k) out[k] = u[k];
}

struct EosParams {
  int kind;  // 0 SC_psi, 1 vdW, 2 RK, 3 PR, 4 CS
  double a, b, R, G, rho0, omega, T_cr;
};

struct FluidModel {
  int kind;  // 0 Newtonian(nu), 1 power law(m, n)
  double nu, m, n;
};

template <class T>
struct Lattice {
  int NX, NY;
  T w[9];
  std::vector<T> f, f2, rho, total_rho, pressure, total_pressure, shear_rate, temp;
  std::vector<T> vel, body_force, scforce, psi;
  std::vector<int32_t> mask, neighbor;
  std::vector<T> tau, tau_sym, tau_antisym, diag;
  T M[81], Minv[81];
  T gravity[2];
  int error = 0;

  Lattice(int nx, int ny) : NX(nx), NY(ny) {
    // lbm.py:44 — weights = (4,1,1,1,1,1/4,1/4,1/4,1/4)/9 in the float type
    const T num[9] = {T(4), T(1), T(1), T(1), T(1), T(0.25), T(0.25), T(0.25), T(0.25)};
    for (int k = 0; k < 9; ++k) w[k] = num[k] / T(9.0);
    size_t n = (size_t)nx * ny;
    f.assign(n * 9, T(0)); f2.assign(n * 9, T(0));
    rho.assign(n, T(0)); total_rho.assign(n, T(0)); pressure.assign(n, T(0));
    total_pressure.assign(n, T(0)); shear_rate.assign(n, T(0)); temp.assign(n, T(0));
    vel.assign(n * 2, T(0)); body_force.assign(n * 2, T(0)); scforce.assign(n * 2, T(0));
    psi.assign((size_t)(nx + 2) * (ny + 2), T(0));
    mask.assign(n, 1);  // lbm.py:74 mask.fill(1)
    neighbor.assign(n * 18, 0);
    tau.assign(n, T(0)); tau_sym.assign(n, T(0)); tau_antisym.assign(n, T(0));
    diag.assign(n * 9, T(0));
    // CollisionEngine.py:273-282 — MRT transform; the inverse is supplied by
    // the caller (the reference rounds numpy's inverse), default exact.
    static const double Mv[81] = {
        1, 1, 1, 1, 1, 1, 1, 1, 1,       -4, -1, -1, -1, -1, 2, 2, 2, 2,
        4, -2, -2, -2, -2, 1, 1, 1, 1,   0, 1, 0, -1, 0, 1, -1, -1, 1,
        0, -2, 0, 2, 0, 1, -1, -1, 1,    0, 0, 1, 0, -1, 1, 1, -1, -1,
        0, 0, -2, 0, 2, 1, 1, -1, -1,    0, 1, -1, 1, -1, 0, 0, 0, 0,
        0, 0, 0, 0, 0, 1, -1, 1, -1};
    for (int q = 0; q < 81; ++q) { M[q] = T(Mv[q]); Minv[q] = T(0); }
    gravity[0] = gravity[1] = T(0);
  }
  size_t id(int i, int j) const { return (size_t)i * NY + j; }
  size_t pid(int i, int j) const { return (size_t)(i + 1) * (NY + 2) + (j + 1); }
  bool inside(int i, int j) const { return i >= 0 && i < NX && j >= 0 && j < NY; }
  T* F(int i, int j) { return &f[id(i, j) * 9]; }
  T* F2(int i, int j) { return &f2[id(i, j) * 9]; }
};

// CollisionEngine.py:15-18 (and BoundaryCondition.py:107-110) — equilibrium
template <class T>
void feq(const T w[9], T ux, T uy, T rho, T out[9]) {
  T uv = ux * ux + uy * uy;
  for (int k = 0; k < 9; ++k) {
    T eu = T(CX[k]) * ux + T(CY[k]) * uy;
    T t = T(1) + T(3) * eu;
    t = t + T(4.5) * eu * eu;
    t = t - T(1.5) * uv;
    out[k] = w[k] * rho * t;
  }
}

// CollisionEngine.py:21-25 — Guo forcing populations
template <class T>
void fforce(const T w[9], T Fx, T Fy, T ux, T uy, T out[9]) {
  T uF = ux * Fx + uy * Fy;
  for (int k = 0; k < 9; ++k) {
    T cF = T(CX[k]) * Fx + T(CY[k]) * Fy;
    T cu = T(CX[k]) * ux + T(CY[k]) * uy;
    T t = T(3) * cF + T(9) * cF * cu;
    t = t - T(3) * uF;
    out[k] = w[k] * t;
  }
}

// CollisionEngine.py:29-34
template <class T>
T clamp_tau(T tau, T lo, T hi) {
  if (tau < lo) tau = lo;
  else if (tau > hi) tau = hi;
  return tau;
}

// FluidModels.py:10-29 — apparent viscosity
template <class T>
T apparent_viscosity(const FluidModel& fm, T shear_rate) {
  if (fm.kind == 0) return T(fm.nu);
  return T(fm.m) * std::pow(shear_rate, T(fm.n - 1.0));
}

// EOS.py — pseudopotential psi(rho, T)
template <class T>
T eos_pressure(const EosParams& e, T d, T Tt) {
  const T a = T(e.a), b = T(e.b), R = T(e.R);
  switch (e.kind) {
    case 1:  // EOS.py:55-58 vdW
      return d * R * Tt / (T(1) - b * d) - a * std::pow(d, T(2));
    case 2:  // EOS.py:66-69 RK
      return d * R * Tt / (T(1) - b * d) - a * std::pow(d, T(2)) / std::sqrt(Tt) / (T(1) + b * d);
    case 3: {  // EOS.py:78-82 PR
      const double om = e.omega;
      const T kap = T(0.37464 + 1.54226 * om - 0.269922 * (om * om));
      T s = T(1) + kap * (T(1) - std::sqrt(Tt / T(e.T_cr)));
      T alpha = s * s;
      T bd = b * d;
      return d * R * Tt / (T(1) - b * d) - a * alpha * (d * d) / (T(1) + T(2) * b * d - bd * bd);
    }
    case 4: {  // EOS.py:90-95 CS
      T b4 = b * d / T(4);
      T aaa = T(1) + b4 + b4 * b4 - b4 * b4 * b4;
      T one = T(1) - b4;
      T bbb = one * one * one;
      return d * R * Tt * aaa / bbb - a * (d * d);
    }
  }
  return T(0);
}

template <class T>
T get_psi(const EosParams& e, T d, T Tt) {
  if (e.kind == 0) {  // EOS.py:45-47 SC_psi
    const T r0 = T(e.rho0);
    return r0 * (T(1) - std::exp(-d / r0));
  }
  // EOS.py:28-32
  T p = eos_pressure(e, d, Tt);
  return std::sqrt(std::fabs(T(6.0 / e.G) * (p - d / T(3))));
}

// ---------------------------------------------------------------- setup
// BoundaryCondition.py:471-475 — strict disc
template <class T>
void mask_circle(Lattice<T>& L, T x, T y, T r) {
  for (int i = 0; i < L.NX; ++i)
    for (int j = 0; j < L.NY; ++j) {
      T dx = T(i) - x, dy = T(j) - y;
      if (dx * dx + dy * dy < r * r) L.mask[L.id(i, j)] = -1;
    }
}

// BoundaryCondition.py:464-469 — open rectangle
template <class T>
void mask_rect(Lattice<T>& L, T xmin, T xmax, T ymin, T ymax) {
  for (int i = 0; i < L.NX; ++i)
    for (int j = 0; j < L.NY; ++j)
      if (T(i) < xmax && T(i) > xmin && T(j) < ymax && T(j) > ymin) L.mask[L.id(i, j)] = -1;
}

// lbm.py:127-142 — pull-source table; solid nodes keep their old entries
template <class T>
void neighbor_classify(Lattice<T>& L) {
#pragma omp parallel for
  for (int i = 0; i < L.NX; ++i)
    for (int j = 0; j < L.NY; ++j) {
      if (L.mask[L.id(i, j)] == -1) continue;
      int32_t* nb = &L.neighbor[L.id(i, j) * 18];
      for (int k = 0; k < 9; ++k) {
        int i2 = i - CX[k], j2 = j - CY[k];
        if (L.inside(i2, j2) && L.mask[L.id(i2, j2)] != -1) { nb[2 * k] = i2; nb[2 * k + 1] = j2; }
        else { nb[2 * k] = -1; nb[2 * k + 1] = -1; }
      }
    }
}

// lbm.py:119-125
template <class T>
void init_lbm(Lattice<T>& L, const int32_t* g, int64_t n) {
#pragma omp parallel for
  for (int64_t m = 0; m < n; ++m) {
    int i = g[2 * m], j = g[2 * m + 1];
    size_t q = L.id(i, j);
    T e[9];
    feq(L.w, L.vel[2 * q], L.vel[2 * q + 1], L.rho[q], e);
    for (int k = 0; k < 9; ++k) { L.F(i, j)[k] = e[k]; L.F2(i, j)[k] = e[k]; }
  }
}

// ---------------------------------------------------------------- moments
// lbm.py:153-164
template <class T>
void density(Lattice<T>& L, const int32_t* g, int64_t n) {
  std::fill(L.total_rho.begin(), L.total_rho.end(), T(0));
  std::fill(L.rho.begin(), L.rho.end(), T(0));
#pragma omp parallel for
  for (int64_t m = 0; m < n; ++m) {
    size_t q = L.id(g[2 * m], g[2 * m + 1]);
    T r = T(0);
    for (int k = 0; k < 9; ++k) r = r + L.f[q * 9 + k];
    L.rho[q] = r;
    L.total_rho[q] = L.total_rho[q] + r;
  }
}

// lbm.py:166-182 — pressure0 (no SC) / pressure1 (single-component SC)
template <class T>
void pressure(Lattice<T>& L, const int32_t* g, int64_t n, int with_sc, double g_coh) {
  std::fill(L.pressure.begin(), L.pressure.end(), T(0));
  const T hg = T(0.5 * g_coh);
#pragma omp parallel for
  for (int64_t m = 0; m < n; ++m) {
    int i = g[2 * m], j = g[2 * m + 1];
    size_t q = L.id(i, j);
    T p;
    if (with_sc) { T ps = L.psi[L.pid(i, j)]; p = (L.rho[q] + hg * (ps * ps)) / T(3); }
    else p = L.rho[q] / T(3);
    L.pressure[q] = L.pressure[q] + p;
    L.total_pressure[q] = L.pressure[q];
  }
}

// lbm.py:215-220
template <class T>
void force_density(Lattice<T>& L, const int32_t* g, int64_t n) {
#pragma omp parallel for
  for (int64_t m = 0; m < n; ++m) {
    size_t q = L.id(g[2 * m], g[2 * m + 1]);
    T s = L.rho[q] / L.total_rho[q];
    L.body_force[2 * q] = L.scforce[2 * q] + s * L.gravity[0];
    L.body_force[2 * q + 1] = L.scforce[2 * q + 1] + s * L.gravity[1];
  }
}

// lbm.py:223-237 body for one node (also BoundaryCondition.py:287-298)
template <class T>
void velocity_node(Lattice<T>& L, size_t q) {
  T vx = T(0), vy = T(0);
  for (int k = 0; k < 9; ++k) {
    vx = vx + L.f[q * 9 + k] * T(CX[k]);
    vy = vy + L.f[q * 9 + k] * T(CY[k]);
  }
  vx = vx + T(0.5) * L.body_force[2 * q];
  vy = vy + T(0.5) * L.body_force[2 * q + 1];
  L.vel[2 * q] = (T(0) + vx) / L.total_rho[q];
  L.vel[2 * q + 1] = (T(0) + vy) / L.total_rho[q];
}

template <class T>
void velocity(Lattice<T>& L, const int32_t* g, int64_t n) {
  std::fill(L.vel.begin(), L.vel.end(), T(0));
#pragma omp parallel for
  for (int64_t m = 0; m < n; ++m) velocity_node(L, L.id(g[2 * m], g[2 * m + 1]));
}

// BoundaryCondition.py:274-280 (OpenBoundary.density) for one node
template <class T>
void density_node(Lattice<T>& L, size_t q) {
  L.total_rho[q] = T(0);
  T r = T(0);
  for (int k = 0; k < 9; ++k) r = r + L.f[q * 9 + k];
  L.rho[q] = r;
  L.total_rho[q] = L.total_rho[q] + r;
}

// ---------------------------------------------------------------- collision
// BGK: CollisionEngine.py:65-70, 72-78, 80-92, 96-110
template <class T>
void bgk_init_tau(Lattice<T>& L, const int32_t* g, int64_t n, double nu) {
  const T tnu = T(nu);
  for (int64_t m = 0; m < n; ++m) L.tau[L.id(g[2 * m], g[2 * m + 1])] = tnu * T(3) + T(0.5);
}

template <class T>
T shear_rate_from_fneq(const T fn[9], T cof) {
  T Sxx = (fn[1] + fn[3] + fn[5] + fn[6] + fn[7] + fn[8]) * cof;
  T Syy = (fn[2] + fn[4] + fn[5] + fn[6] + fn[7] + fn[8]) * cof;
  T Sxy = (fn[5] - fn[6] + fn[7] - fn[8]) * cof;
  return std::sqrt(T(2) * (Sxx * Sxx + Syy * Syy + T(2) * (Sxy * Sxy)));
}

// BGK/TRT shear_rate: tau_field is tau (BGK) or tau_sym (TRT)
template <class T>
void shear_rate_tau(Lattice<T>& L, const int32_t* g, int64_t n, const std::vector<T>& tau_field) {
#pragma omp parallel for
  for (int64_t m = 0; m < n; ++m) {
    size_t q = L.id(g[2 * m], g[2 * m + 1]);
    T e[9], fn[9];
    feq(L.w, L.vel[2 * q], L.vel[2 * q + 1], L.rho[q], e);
    for (int k = 0; k < 9; ++k) fn[k] = L.f[q * 9 + k] - e[k];
    T cof = T(-1.5) / L.rho[q] / tau_field[q];
    L.shear_rate[q] = shear_rate_from_fneq(fn, cof);
  }
}

template <class T>
void bgk_relaxation_time(Lattice<T>& L, const int32_t* g, int64_t n, FluidModel fm, double lo, double hi) {
#pragma omp parallel for
  for (int64_t m = 0; m < n; ++m) {
    size_t q = L.id(g[2 * m], g[2 * m + 1]);
    T t = apparent_viscosity(fm, L.shear_rate[q]) * T(3) + T(0.5);
    L.tau[q] = clamp_tau(t, T(lo), T(hi));
  }
}

template <class T>
void bgk_apply(Lattice<T>& L, const int32_t* g, int64_t n) {
#pragma omp parallel for
  for (int64_t m = 0; m < n; ++m) {
    size_t q = L.id(g[2 * m], g[2 * m + 1]);
    T omega = T(1) / L.tau[q];
    T ux = L.vel[2 * q], uy = L.vel[2 * q + 1];
    T e[9], fo[9];
    feq(L.w, ux, uy, L.rho[q], e);
    fforce(L.w, L.body_force[2 * q], L.body_force[2 * q + 1], ux, uy, fo);
    const T* f = &L.f[q * 9];
    T* f2 = &L.f2[q * 9];
    T cf = T(1) - T(0.5) * omega;
    for (int k = 0; k < 9; ++k) {
      T co = (-omega) * (f[k] - e[k]);
      T ft = cf * fo[k];
      f2[k] = f[k] + co + ft;
    }
  }
}

// TRT: CollisionEngine.py:149-155, 157-164, 166-178, 181-245
template <class T>
void trt_init_tau(Lattice<T>& L, const int32_t* g, int64_t n, double nu, double magic) {
  const T tnu = T(nu), mg = T(magic);
  for (int64_t m = 0; m < n; ++m) {
    size_t q = L.id(g[2 * m], g[2 * m + 1]);
    L.tau_sym[q] = tnu * T(3) + T(0.5);
    L.tau_antisym[q] = mg / (L.tau_sym[q] - T(0.5)) + T(0.5);
  }
}

template <class T>
void trt_relaxation_time(Lattice<T>& L, const int32_t* g, int64_t n, FluidModel fm, double magic,
                         double lo, double hi) {
  const T mg = T(magic);
#pragma omp parallel for
  for (int64_t m = 0; m < n; ++m) {
    size_t q = L.id(g[2 * m], g[2 * m + 1]);
    T t = apparent_viscosity(fm, L.shear_rate[q]) * T(3) + T(0.5);
    L.tau_sym[q] = clamp_tau(t, T(lo), T(hi));
    L.tau_antisym[q] = mg / (L.tau_sym[q] - T(0.5)) + T(0.5);
  }
}

template <class T>
void sym_part(const T v[9], T s[9]) {
  s[0] = v[0];
  s[1] = (v[1] + v[3]) / T(2);
  s[2] = (v[2] + v[4]) / T(2);
  s[3] = s[1];
  s[4] = s[2];
  s[5] = (v[5] + v[7]) / T(2);
  s[6] = (v[6] + v[8]) / T(2);
  s[7] = s[5];
  s[8] = s[6];
}

template <class T>
void trt_apply(Lattice<T>& L, const int32_t* g, int64_t n) {
#pragma omp parallel for
  for (int64_t m = 0; m < n; ++m) {
    size_t q = L.id(g[2 * m], g[2 * m + 1]);
    T os = T(1) / L.tau_sym[q];
    T oa = T(1) / L.tau_antisym[q];
    T ux = L.vel[2 * q], uy = L.vel[2 * q + 1];
    T e[9], fo[9], fs[9], es[9], ffs[9];
    feq(L.w, ux, uy, L.rho[q], e);
    fforce(L.w, L.body_force[2 * q], L.body_force[2 * q + 1], ux, uy, fo);
    const T* f = &L.f[q * 9];
    T* f2 = &L.f2[q * 9];
    sym_part(f, fs);
    sym_part(e, es);
    sym_part(fo, ffs);
    T cs = T(1) - T(0.5) * os, ca = T(1) - T(0.5) * oa;
    for (int k = 0; k < 9; ++k) {
      T fa = f[k] - fs[k], ea = e[k] - es[k], foa = fo[k] - ffs[k];
      T co = (-os) * (fs[k] - es[k]) - oa * (fa - ea);
      T ft = cs * ffs[k] + ca * foa;
      f2[k] = f[k] + co + ft;
    }
  }
}

// MRT: CollisionEngine.py:301-318, 322-329, 332-377, 379-451
template <class T>
void mrt_init_tau(Lattice<T>& L, const int32_t* g, int64_t n, double nu, double nu_bulk, double lo,
                  double hi) {
  std::fill(L.diag.begin(), L.diag.end(), T(1));
  for (int64_t m = 0; m < n; ++m) {
    size_t q = L.id(g[2 * m], g[2 * m + 1]);
    T* d = &L.diag[q * 9];
    T t = clamp_tau(T(nu) * T(3) + T(0.5), T(lo), T(hi));
    d[7] = d[8] = T(1) / t;
    T tb = clamp_tau(T(nu_bulk) * T(3) + T(0.5), T(lo), T(hi));
    d[1] = T(1) / tb;
    d[0] = T(0);
    d[3] = T(0);
    d[5] = T(0);
  }
}

template <class T>
void mrt_mf(const T M[81], const T f[9], T m[9]) {
  for (int a = 0; a < 9; ++a) {
    T s = T(0);
    for (int b = 0; b < 9; ++b) s = s + M[a * 9 + b] * f[b];
    m[a] = s;
  }
}

template <class T>
void mrt_relaxation_time(Lattice<T>& L, const int32_t* g, int64_t n, FluidModel fm, double lo, double hi) {
#pragma omp parallel for
  for (int64_t m = 0; m < n; ++m) {
    size_t q = L.id(g[2 * m], g[2 * m + 1]);
    T t = clamp_tau(apparent_viscosity(fm, L.shear_rate[q]) * T(3) + T(0.5), T(lo), T(hi));
    L.diag[q * 9 + 7] = L.diag[q * 9 + 8] = T(1) / t;
  }
}

template <class T>
void mrt_shear_rate(Lattice<T>& L, const int32_t* g, int64_t n) {
#pragma omp parallel for
  for (int64_t m = 0; m < n; ++m) {
    size_t q = L.id(g[2 * m], g[2 * m + 1]);
    T e[9], fn[9], mn[9], smn[9], mneq[9];
    feq(L.w, L.vel[2 * q], L.vel[2 * q + 1], L.rho[q], e);
    for (int k = 0; k < 9; ++k) fn[k] = L.f[q * 9 + k] - e[k];
    mrt_mf(L.M, fn, mn);
    for (int k = 0; k < 9; ++k) smn[k] = L.diag[q * 9 + k] * mn[k];
    mrt_mf(L.Minv, smn, mneq);
    T cof = T(-1.5) / L.rho[q];
    L.shear_rate[q] = shear_rate_from_fneq(mneq, cof);
  }
}

template <class T>
void mrt_apply(Lattice<T>& L, const int32_t* g, int64_t n) {
#pragma omp parallel for
  for (int64_t m = 0; m < n; ++m) {
    size_t q = L.id(g[2 * m], g[2 * m + 1]);
    const T* f = &L.f[q * 9];
    const T* d = &L.diag[q * 9];
    T mm[9], meq[9], mfo[9], m2[9];
    mrt_mf(L.M, f, mm);
    T jx = L.vel[2 * q], jy = L.vel[2 * q + 1], r = L.rho[q];
    T u2 = jx * jx + jy * jy;
    meq[0] = T(1);
    meq[1] = T(-2) + T(3) * u2;
    meq[2] = T(1) - T(3) * u2;
    meq[3] = jx;
    meq[4] = -jx;
    meq[5] = jy;
    meq[6] = -jy;
    meq[7] = jx * jx - jy * jy;
    meq[8] = jx * jy;
    for (int k = 0; k < 9; ++k) meq[k] = meq[k] * r;
    T Fx = L.body_force[2 * q], Fy = L.body_force[2 * q + 1];
    T Fu = Fx * jx + Fy * jy;
    mfo[0] = T(0);
    mfo[1] = T(6) * Fu;
    mfo[2] = T(-6) * Fu;
    mfo[3] = Fx;
    mfo[4] = -Fx;
    mfo[5] = Fy;
    mfo[6] = -Fy;
    mfo[7] = T(2) * (Fx * jx - Fy * jy);
    mfo[8] = Fy * jx + Fx * jy;
    for (int k = 0; k < 9; ++k) {
      T a = d[k] * (mm[k] - meq[k]);
      T b = (T(1) - d[k] / T(2)) * mfo[k];
      m2[k] = mm[k] - a + b;
    }
    mrt_mf(L.Minv, m2, &L.f2[q * 9]);
  }
}

// ---------------------------------------------------------------- Shan-Chen
// ExternalForce.py:42-47
template <class T>
void sc_update_psi(Lattice<T>& L, const int32_t* g, int64_t n, EosParams e) {
#pragma omp parallel for
  for (int64_t m = 0; m < n; ++m) {
    int i = g[2 * m], j = g[2 * m + 1];
    L.psi[L.pid(i, j)] = get_psi(e, L.rho[L.id(i, j)], L.temp[L.id(i, j)]);
  }
}

// SCBoundaryCondition.py:126-144 — periodic psi halo, LR then BT
template <class T>
void psi_periodic_lr(Lattice<T>& L) {
  for (int y = -1; y <= L.NY; ++y) {
    L.psi[L.pid(-1, y)] = L.psi[L.pid(L.NX - 1, y)];
    L.psi[L.pid(L.NX, y)] = L.psi[L.pid(0, y)];
  }
}
template <class T>
void psi_periodic_bt(Lattice<T>& L) {
  for (int x = -1; x <= L.NX; ++x) {
    L.psi[L.pid(x, -1)] = L.psi[L.pid(x, L.NY - 1)];
    L.psi[L.pid(x, L.NY)] = L.psi[L.pid(x, 0)];
  }
}

// SCBoundaryCondition.py:113-123 — FixedPsi
template <class T>
void psi_fixed(Lattice<T>& L, const int32_t* g, int64_t n, double value) {
  for (int64_t m = 0; m < n; ++m) L.psi[L.pid(g[2 * m], g[2 * m + 1])] = T(value);
}

// SCBoundaryCondition.py:19-110 — open psi boundaries on a group of psi
// nodes (halo coordinates allowed): kind 0 OpenNeumannPsi, 1
// OpenConvective1orderPsi, 2 OpenConvective2orderPsi, 3
// OpenExtrapolationPsi.  The convective kinds first average the velocity of
// the neighbours x - c_dir over the group, in group order (serially), and
// take lambda = |U|.
template <class T>
void psi_open(Lattice<T>& L, const int32_t* g, int64_t n, int kind, int dir) {
  const int cx = CX[dir], cy = CY[dir];
  T lam = T(0);
  if (kind == 1 || kind == 2) {
    T Ux = T(0), Uy = T(0);
    for (int64_t m = 0; m < n; ++m) {
      size_t q2 = L.id(g[2 * m] - cx, g[2 * m + 1] - cy);
      Ux = Ux + L.vel[2 * q2];
      Uy = Uy + L.vel[2 * q2 + 1];
    }
    Ux = Ux / T(n);
    Uy = Uy / T(n);
    lam = T(1) * std::sqrt(Ux * Ux + Uy * Uy);
  }
  for (int64_t m = 0; m < n; ++m) {
    const int i = g[2 * m], j = g[2 * m + 1];
    const size_t p = L.pid(i, j), p2 = L.pid(i - cx, j - cy), p3 = L.pid(i - 2 * cx, j - 2 * cy);
    if (kind == 0) L.psi[p] = L.psi[p2];
    else if (kind == 1) L.psi[p] = (L.psi[p] + lam * L.psi[p2]) / (T(1) + lam);
    else if (kind == 2)
      L.psi[p] = (L.psi[p] + T(2) * lam * L.psi[p2] - T(0.5) * lam * L.psi[p3]) / (T(1) + T(1.5) * lam);
    else L.psi[p] = T(2) * L.psi[p2] - L.psi[p3];
  }
}

// SC force at one node (ExternalForce.py:50-63 and BoundaryCondition.py:301-312)
template <class T>
void sc_force_node(Lattice<T>& L, int i, int j, T g_coh) {
  T Fx = T(0), Fy = T(0);
  for (int k = 1; k < 9; ++k) {
    T wcx = L.w[k] * T(CX[k]), wcy = L.w[k] * T(CY[k]);
    T p = L.psi[L.pid(i + CX[k], j + CY[k])];
    Fx = Fx + wcx * p;
    Fy = Fy + wcy * p;
  }
  T s = (-g_coh) * L.psi[L.pid(i, j)];
  Fx = Fx * s;
  Fy = Fy * s;
  size_t q = L.id(i, j);
  L.scforce[2 * q] = T(0) + Fx;
  L.scforce[2 * q + 1] = T(0) + Fy;
}

// ExternalForce.py:50-63
template <class T>
void sc_force(Lattice<T>& L, const int32_t* g, int64_t n, double g_coh) {
  std::fill(L.scforce.begin(), L.scforce.end(), T(0));
  const T gc = T(g_coh);
#pragma omp parallel for
  for (int64_t m = 0; m < n; ++m) sc_force_node(L, g[2 * m], g[2 * m + 1], gc);
}

// ---------------------------------------------------------------- stream carriers
// BoundaryCondition.py:424-432
template <class T>
void bc_periodic(Lattice<T>& L, const int32_t* g, int64_t n) {
#pragma omp parallel for
  for (int64_t m = 0; m < n; ++m) {
    int i = g[2 * m], j = g[2 * m + 1];
    for (int k = 0; k < 9; ++k) {
      int x2 = (i - CX[k] + L.NX) % L.NX, y2 = (j - CY[k] + L.NY) % L.NY;
      L.F(i, j)[k] = L.F2(x2, y2)[k];
    }
  }
}

// BoundaryCondition.py:440-449; a -1 entry is an out-of-range read in the
// reference (undefined) and is flagged instead of being performed
template <class T>
void bc_inside(Lattice<T>& L, const int32_t* g, int64_t n) {
  int err = 0;
#pragma omp parallel for reduction(| : err)
  for (int64_t m = 0; m < n; ++m) {
    int i = g[2 * m], j = g[2 * m + 1];
    const int32_t* nb = &L.neighbor[L.id(i, j) * 18];
    for (int k = 0; k < 9; ++k) {
      if (nb[2 * k] < 0) { err |= 1; continue; }
      L.F(i, j)[k] = L.F2(nb[2 * k], nb[2 * k + 1])[k];
    }
  }
  L.error |= err;
}

// BoundaryCondition.py:244-259
template <class T>
void bc_bounceback(Lattice<T>& L, const int32_t* g, int64_t n) {
#pragma omp parallel for
  for (int64_t m = 0; m < n; ++m) {
    int i = g[2 * m], j = g[2 * m + 1];
    const int32_t* nb = &L.neighbor[L.id(i, j) * 18];
    for (int k = 0; k < 9; ++k) {
      if (nb[2 * k] != -1) L.F(i, j)[k] = L.F2(nb[2 * k], nb[2 * k + 1])[k];
      else L.F(i, j)[k] = L.F2(i, j)[OPP[k]];
    }
  }
}

// ---------------------------------------------------------------- velocity/pressure BCs
// BoundaryCondition.py:119-129
template <class T>
T rhow(int dir, T vx, T vy, const T* f) {
  if (dir == 2) return T(1) / (T(1) + vy) * (f[0] + f[1] + f[3] + T(2) * (f[2] + f[5] + f[6]));
  if (dir == 4) return T(1) / (T(1) - vy) * (f[0] + f[1] + f[3] + T(2) * (f[4] + f[7] + f[8]));
  if (dir == 1) return T(1) / (T(1) + vx) * (f[0] + f[2] + f[4] + T(2) * (f[1] + f[5] + f[8]));
  if (dir == 3) return T(1) / (T(1) - vx) * (f[0] + f[2] + f[4] + T(2) * (f[3] + f[6] + f[7]));
  return T(0);
}

// uvel: per-node (n x 2) velocities in the float type of the lattice
// BoundaryCondition.py:85-102 — VelocityBB
template <class T>
void bc_velocity_bb(Lattice<T>& L, const int32_t* g, int64_t n, int dir, const T* uvel) {
  int un[3];
  unknowns(dir, un);
  for (int64_t m = 0; m < n; ++m) {
    int i = g[2 * m], j = g[2 * m + 1];
    size_t q = L.id(i, j);
    T Ux = uvel[2 * m], Uy = uvel[2 * m + 1];
    T rw = L.rho[q];
    for (int t = 0; t < 3; ++t) {
      int d = un[t];
      T cv = T(CX[d]) * Ux + T(CY[d]) * Uy;
      L.f[q * 9 + d] = L.f[q * 9 + d] + T(6) * L.w[d] * rw * cv;
    }
  }
}

// BoundaryCondition.py:137-147 — VelocityEquilibrium
template <class T>
void bc_velocity_eq(Lattice<T>& L, const int32_t* g, int64_t n, int dir, const T* uvel) {
  for (int64_t m = 0; m < n; ++m) {
    size_t q = L.id(g[2 * m], g[2 * m + 1]);
    T Ux = uvel[2 * m], Uy = uvel[2 * m + 1];
    L.vel[2 * q] = Ux;
    L.vel[2 * q + 1] = Uy;
    L.rho[q] = rhow(dir, Ux, Uy, &L.f[q * 9]);
    feq(L.w, L.vel[2 * q], L.vel[2 * q + 1], L.rho[q], &L.f[q * 9]);
  }
}

// BoundaryCondition.py:112-116 + 154-166 — VelocityNEEM
template <class T>
void bc_velocity_neem(Lattice<T>& L, const int32_t* g, int64_t n, int dir, const T* uvel) {
  for (int64_t m = 0; m < n; ++m) {
    int i = g[2 * m], j = g[2 * m + 1];
    int i2 = i - CX[dir], j2 = j - CY[dir];
    size_t q = L.id(i, j), q2 = L.id(i2, j2);
    T Ux = uvel[2 * m], Uy = uvel[2 * m + 1];
    L.vel[2 * q] = Ux;
    L.vel[2 * q + 1] = Uy;
    L.rho[q] = rhow(dir, Ux, Uy, &L.f[q * 9]);
    T eb[9], ef[9];
    feq(L.w, L.vel[2 * q], L.vel[2 * q + 1], L.rho[q], eb);
    feq(L.w, L.vel[2 * q2], L.vel[2 * q2 + 1], L.rho[q2], ef);
    for (int k = 0; k < 9; ++k) L.f[q * 9 + k] = eb[k] + L.f[q2 * 9 + k] - ef[k];
  }
}

// BoundaryCondition.py:182-205 — PressureABC
template <class T>
void bc_pressure_abc(Lattice<T>& L, const int32_t* g, int64_t n, int dir, double rho_value) {
  int un[3];
  unknowns(dir, un);
  const T rw = T(rho_value);
  for (int64_t m = 0; m < n; ++m) {
    int i = g[2 * m], j = g[2 * m + 1];
    size_t q = L.id(i, j), q2 = L.id(i - CX[dir], j - CY[dir]);
    T ux = T(1.5) * L.vel[2 * q] - T(0.5) * L.vel[2 * q2];
    T uy = T(1.5) * L.vel[2 * q + 1] - T(0.5) * L.vel[2 * q2 + 1];
    L.vel[2 * q] = ux;
    L.vel[2 * q + 1] = uy;
    L.total_rho[q] = rw;
    T uw2 = ux * ux + uy * uy;
    T ft[9];
    for (int k = 0; k < 9; ++k) {
      T cu = T(CX[k]) * ux + T(CY[k]) * uy;
      T t = T(1) + T(4.5) * cu * cu;
      t = t - T(1.5) * uw2;
      ft[k] = -L.f[q * 9 + k] + T(2) * L.w[k] * rw * t;
    }
    for (int t = 0; t < 3; ++t) L.f[q * 9 + un[t]] = ft[un[t]];
  }
}

// BoundaryCondition.py:215-226 — PressureNEEM (rho_value only reaches total_rho)
template <class T>
void bc_pressure_neem(Lattice<T>& L, const int32_t* g, int64_t n, int dir, double rho_value) {
  int un[3];
  unknowns(dir, un);
  for (int64_t m = 0; m < n; ++m) {
    int i = g[2 * m], j = g[2 * m + 1];
    size_t q = L.id(i, j), q2 = L.id(i - CX[dir], j - CY[dir]);
    L.vel[2 * q] = L.vel[2 * q2];
    L.vel[2 * q + 1] = L.vel[2 * q2 + 1];
    L.total_rho[q] = T(rho_value);
    T eb[9], ef[9];
    feq(L.w, L.vel[2 * q], L.vel[2 * q + 1], L.rho[q], eb);
    feq(L.w, L.vel[2 * q2], L.vel[2 * q2 + 1], L.rho[q2], ef);
    for (int t = 0; t < 3; ++t) {
      int d = un[t];
      L.f[q * 9 + d] = eb[d] + L.f[q2 * 9 + d] - ef[d];
    }
  }
}

// ---------------------------------------------------------------- open BCs
// BoundaryCondition.py:321-334
template <class T>
void bc_open_neumann(Lattice<T>& L, const int32_t* g, int64_t n, int dir) {
  int un[3];
  unknowns(dir, un);
  for (int64_t m = 0; m < n; ++m) {
    int i = g[2 * m], j = g[2 * m + 1];
    size_t q = L.id(i, j), q2 = L.id(i - CX[dir], j - CY[dir]);
    for (int t = 0; t < 3; ++t) L.f[q * 9 + un[t]] = L.f[q2 * 9 + un[t]];
    density_node(L, q);
    velocity_node(L, q);
  }
}

// BoundaryCondition.py:342-359
template <class T>
void bc_open_conv1(Lattice<T>& L, const int32_t* g, int64_t n, int dir) {
  int un[3];
  unknowns(dir, un);
  for (int64_t m = 0; m < n; ++m) {
    int i = g[2 * m], j = g[2 * m + 1];
    size_t q = L.id(i, j), q2 = L.id(i - CX[dir], j - CY[dir]);
    T Ux = L.vel[2 * q2], Uy = L.vel[2 * q2 + 1];
    T lam = T(1) * std::sqrt(Ux * Ux + Uy * Uy);
    for (int t = 0; t < 3; ++t) {
      int d = un[t];
      L.f[q * 9 + d] = (L.f[q * 9 + d] + lam * L.f[q2 * 9 + d]) / (T(1) + lam);
    }
    density_node(L, q);
    velocity_node(L, q);
  }
}

// BoundaryCondition.py:367-390 (needs the Shan-Chen field)
template <class T>
void bc_open_conv2(Lattice<T>& L, const int32_t* g, int64_t n, int dir, double g_coh, EosParams e) {
  int un[3];
  unknowns(dir, un);
  const T gc = T(g_coh);
  for (int it = 0; it < 3; ++it)
    for (int64_t m = 0; m < n; ++m) {
      int i = g[2 * m], j = g[2 * m + 1];
      int i2 = i - CX[dir], j2 = j - CY[dir], i3 = i - 2 * CX[dir], j3 = j - 2 * CY[dir];
      size_t q = L.id(i, j), q2 = L.id(i2, j2), q3 = L.id(i3, j3);
      sc_force_node(L, i2, j2, gc);
      T s = L.rho[q2] / L.total_rho[q2];
      L.body_force[2 * q2] = L.scforce[2 * q2] + s * L.gravity[0];
      L.body_force[2 * q2 + 1] = L.scforce[2 * q2 + 1] + s * L.gravity[1];
      velocity_node(L, q2);
      T Ux = L.vel[2 * q2], Uy = L.vel[2 * q2 + 1];
      T lam = T(1) * std::sqrt(Ux * Ux + Uy * Uy);
      for (int t = 0; t < 3; ++t) {
        int d = un[t];
        L.f[q * 9 + d] = (L.f[q * 9 + d] + T(2) * lam * L.f[q2 * 9 + d] - T(0.5) * lam * L.f[q3 * 9 + d]) /
                         (T(1) + T(1.5) * lam);
      }
      density_node(L, q);
      L.psi[L.pid(i, j)] = get_psi(e, L.rho[q], L.temp[q]);
    }
}

// BoundaryCondition.py:400-411
template <class T>
void bc_open_extrap(Lattice<T>& L, const int32_t* g, int64_t n, int dir) {
  int un[3];
  unknowns(dir, un);
  for (int64_t m = 0; m < n; ++m) {
    int i = g[2 * m], j = g[2 * m + 1];
    int i2 = i - CX[dir], j2 = j - CY[dir];
    size_t q = L.id(i, j), q2 = L.id(i2, j2), q3 = L.id(i2 - CX[dir], j2 - CY[dir]);
    for (int t = 0; t < 3; ++t) {
      int d = un[t];
      L.f[q * 9 + d] = T(2) * L.f[q2 * 9 + d] - L.f[q3 * 9 + d];
    }
  }
}

// ---------------------------------------------------------------- handle
struct Handle {
  int dbl;
  Lattice<float>* lf = nullptr;
  Lattice<double>* ld = nullptr;
};

}  // namespace

#define DISPATCH(h, CALL)                 \
  do {                                    \
    if ((h)->dbl) { auto& L = *(h)->ld; CALL; } \
    else { auto& L = *(h)->lf; CALL; }    \
  } while (0)

template <class T>
static void* field_of(Lattice<T>& L, const std::string& s, int64_t* c) {
  struct Entry { const char* nm; void* ptr; size_t n; };
  const Entry tab[] = {
      {"f", L.f.data(), L.f.size()}, {"f2", L.f2.data(), L.f2.size()},
      {"rho", L.rho.data(), L.rho.size()}, {"total_rho", L.total_rho.data(), L.total_rho.size()},
      {"pressure", L.pressure.data(), L.pressure.size()},
      {"total_pressure", L.total_pressure.data(), L.total_pressure.size()},
      {"shear_rate", L.shear_rate.data(), L.shear_rate.size()}, {"T", L.temp.data(), L.temp.size()},
      {"vel", L.vel.data(), L.vel.size()}, {"body_force", L.body_force.data(), L.body_force.size()},
      {"SCforce", L.scforce.data(), L.scforce.size()}, {"psi", L.psi.data(), L.psi.size()},
      {"mask", L.mask.data(), L.mask.size()}, {"neighbor", L.neighbor.data(), L.neighbor.size()},
      {"tau", L.tau.data(), L.tau.size()}, {"tau_sym", L.tau_sym.data(), L.tau_sym.size()},
      {"tau_antisym", L.tau_antisym.data(), L.tau_antisym.size()},
      {"diag", L.diag.data(), L.diag.size()}, {"M", L.M, 81}, {"M_inverse", L.Minv, 81},
      {"weights", L.w, 9}, {"gravity", L.gravity, 2}};
  for (const Entry& e : tab)
    if (s == e.nm) { *c = (int64_t)e.n; return e.ptr; }
  *c = 0;
  return nullptr;
}

extern "C" {

// Pointer to a named field and its element count (float or double per the
// handle's precision; "mask"/"neighbor" are int32).
void* orc_field(void* p, const char* name, int64_t* count) {
  Handle* h = (Handle*)p;
  if (h->dbl) return field_of(*h->ld, std::string(name), count);
  return field_of(*h->lf, std::string(name), count);
}

void* orc_create(int nx, int ny, int dbl) {
  Handle* h = new Handle();
  h->dbl = dbl;
  if (dbl) h->ld = new Lattice<double>(nx, ny);
  else h->lf = new Lattice<float>(nx, ny);
  return h;
}

void orc_destroy(void* p) {
  Handle* h = (Handle*)p;
  delete h->lf;
  delete h->ld;
  delete h;
}

// Pointer to a named field and its element count (float or double per the
// handle's precision; "mask"/"neighbor" are int32).
int orc_error(void* p) {
  Handle* h = (Handle*)p;
  int e = 0;
  DISPATCH(h, e = L.error);
  return e;
}

void orc_mask_circle(void* p, double x, double y, double r) {
  Handle* h = (Handle*)p;
  if (h->dbl) mask_circle(*h->ld, x, y, r);
  else mask_circle(*h->lf, (float)x, (float)y, (float)r);
}
void orc_mask_rect(void* p, double x0, double x1, double y0, double y1) {
  Handle* h = (Handle*)p;
  if (h->dbl) mask_rect(*h->ld, x0, x1, y0, y1);
  else mask_rect(*h->lf, (float)x0, (float)x1, (float)y0, (float)y1);
}
void orc_neighbor_classify(void* p) { DISPATCH((Handle*)p, neighbor_classify(L)); }
void orc_init_lbm(void* p, const int32_t* g, int64_t n) { DISPATCH((Handle*)p, init_lbm(L, g, n)); }
void orc_density(void* p, const int32_t* g, int64_t n) { DISPATCH((Handle*)p, density(L, g, n)); }
void orc_pressure(void* p, const int32_t* g, int64_t n, int with_sc, double g_coh) {
  DISPATCH((Handle*)p, pressure(L, g, n, with_sc, g_coh));
}
void orc_force_density(void* p, const int32_t* g, int64_t n) { DISPATCH((Handle*)p, force_density(L, g, n)); }
void orc_velocity(void* p, const int32_t* g, int64_t n) { DISPATCH((Handle*)p, velocity(L, g, n)); }

static FluidModel fm_of(int kind, double nu, double m, double nexp) {
  FluidModel fm;
  fm.kind = kind; fm.nu = nu; fm.m = m; fm.n = nexp;
  return fm;
}

void orc_bgk_init_tau(void* p, const int32_t* g, int64_t n, double nu) {
  DISPATCH((Handle*)p, bgk_init_tau(L, g, n, nu));
}
void orc_bgk_shear_rate(void* p, const int32_t* g, int64_t n) {
  DISPATCH((Handle*)p, shear_rate_tau(L, g, n, L.tau));
}
void orc_bgk_relaxation_time(void* p, const int32_t* g, int64_t n, int fk, double nu, double m, double ne,
                             double lo, double hi) {
  DISPATCH((Handle*)p, bgk_relaxation_time(L, g, n, fm_of(fk, nu, m, ne), lo, hi));
}
void orc_bgk_apply(void* p, const int32_t* g, int64_t n) { DISPATCH((Handle*)p, bgk_apply(L, g, n)); }

void orc_trt_init_tau(void* p, const int32_t* g, int64_t n, double nu, double magic) {
  DISPATCH((Handle*)p, trt_init_tau(L, g, n, nu, magic));
}
void orc_trt_shear_rate(void* p, const int32_t* g, int64_t n) {
  DISPATCH((Handle*)p, shear_rate_tau(L, g, n, L.tau_sym));
}
void orc_trt_relaxation_time(void* p, const int32_t* g, int64_t n, int fk, double nu, double m, double ne,
                             double magic, double lo, double hi) {
  DISPATCH((Handle*)p, trt_relaxation_time(L, g, n, fm_of(fk, nu, m, ne), magic, lo, hi));
}
void orc_trt_apply(void* p, const int32_t* g, int64_t n) { DISPATCH((Handle*)p, trt_apply(L, g, n)); }

void orc_mrt_init_tau(void* p, const int32_t* g, int64_t n, double nu, double nub, double lo, double hi) {
  DISPATCH((Handle*)p, mrt_init_tau(L, g, n, nu, nub, lo, hi));
}
void orc_mrt_shear_rate(void* p, const int32_t* g, int64_t n) { DISPATCH((Handle*)p, mrt_shear_rate(L, g, n)); }
void orc_mrt_relaxation_time(void* p, const int32_t* g, int64_t n, int fk, double nu, double m, double ne,
                             double lo, double hi) {
  DISPATCH((Handle*)p, mrt_relaxation_time(L, g, n, fm_of(fk, nu, m, ne), lo, hi));
}
void orc_mrt_apply(void* p, const int32_t* g, int64_t n) { DISPATCH((Handle*)p, mrt_apply(L, g, n)); }

static EosParams eos_of(const double* e) {
  EosParams p;
  p.kind = (int)e[0]; p.a = e[1]; p.b = e[2]; p.R = e[3]; p.G = e[4]; p.rho0 = e[5]; p.omega = e[6];
  p.T_cr = e[7];
  return p;
}

// eos: 8 doubles {kind, a, b, R, G, rho0, omega, T_cr}
void orc_sc_update_psi(void* p, const int32_t* g, int64_t n, const double* eos) {
  DISPATCH((Handle*)p, sc_update_psi(L, g, n, eos_of(eos)));
}
void orc_sc_force(void* p, const int32_t* g, int64_t n, double g_coh) {
  DISPATCH((Handle*)p, sc_force(L, g, n, g_coh));
}
void orc_psi_periodic_lr(void* p) { DISPATCH((Handle*)p, psi_periodic_lr(L)); }
void orc_psi_periodic_bt(void* p) { DISPATCH((Handle*)p, psi_periodic_bt(L)); }
void orc_psi_fixed(void* p, const int32_t* g, int64_t n, double v) { DISPATCH((Handle*)p, psi_fixed(L, g, n, v)); }
void orc_psi_open(void* p, const int32_t* g, int64_t n, int kind, int dir) {
  DISPATCH((Handle*)p, psi_open(L, g, n, kind, dir));
}

double orc_get_psi(const double* eos, double rho, double T, int dbl) {
  if (dbl) return get_psi(eos_of(eos), rho, T);
  return (double)get_psi(eos_of(eos), (float)rho, (float)T);
}

void orc_bc_periodic(void* p, const int32_t* g, int64_t n) { DISPATCH((Handle*)p, bc_periodic(L, g, n)); }
void orc_bc_inside(void* p, const int32_t* g, int64_t n) { DISPATCH((Handle*)p, bc_inside(L, g, n)); }
void orc_bc_bounceback(void* p, const int32_t* g, int64_t n) { DISPATCH((Handle*)p, bc_bounceback(L, g, n)); }

// uvel points to n*2 values of the lattice's float type
void orc_bc_velocity_bb(void* p, const int32_t* g, int64_t n, int dir, const void* uvel) {
  Handle* h = (Handle*)p;
  if (h->dbl) bc_velocity_bb(*h->ld, g, n, dir, (const double*)uvel);
  else bc_velocity_bb(*h->lf, g, n, dir, (const float*)uvel);
}
void orc_bc_velocity_eq(void* p, const int32_t* g, int64_t n, int dir, const void* uvel) {
  Handle* h = (Handle*)p;
  if (h->dbl) bc_velocity_eq(*h->ld, g, n, dir, (const double*)uvel);
  else bc_velocity_eq(*h->lf, g, n, dir, (const float*)uvel);
}
void orc_bc_velocity_neem(void* p, const int32_t* g, int64_t n, int dir, const void* uvel) {
  Handle* h = (Handle*)p;
  if (h->dbl) bc_velocity_neem(*h->ld, g, n, dir, (const double*)uvel);
  else bc_velocity_neem(*h->lf, g, n, dir, (const float*)uvel);
}
void orc_bc_pressure_abc(void* p, const int32_t* g, int64_t n, int dir, double rho) {
  DISPATCH((Handle*)p, bc_pressure_abc(L, g, n, dir, rho));
}
void orc_bc_pressure_neem(void* p, const int32_t* g, int64_t n, int dir, double rho) {
  DISPATCH((Handle*)p, bc_pressure_neem(L, g, n, dir, rho));
}
void orc_bc_open_neumann(void* p, const int32_t* g, int64_t n, int dir) {
  DISPATCH((Handle*)p, bc_open_neumann(L, g, n, dir));
}
void orc_bc_open_conv1(void* p, const int32_t* g, int64_t n, int dir) {
  DISPATCH((Handle*)p, bc_open_conv1(L, g, n, dir));
}
void orc_bc_open_conv2(void* p, const int32_t* g, int64_t n, int dir, double g_coh, const double* eos) {
  DISPATCH((Handle*)p, bc_open_conv2(L, g, n, dir, g_coh, eos_of(eos)));
}
void orc_bc_open_extrap(void* p, const int32_t* g, int64_t n, int dir) {
  DISPATCH((Handle*)p, bc_open_extrap(L, g, n, dir));
}

}  // extern "C"
