// FP64 evaluation of a hit and its polish, shared by the final check of the
// batched / learned engines (ho_check.cuh) and the plain kernel.
//
// The FP32 solves stop on the reference's own criteria (inverse-map step
// below 1e-5, surface residual below 1e-4, isosurface |f| below 1e-5). The
// check re-evaluates the returned point in FP64 from the element's
// coefficients: the position x(xi) against o + t d, and for an isosurface
// hit the field u(xi) against the isovalue.
//
// The polish: those stopping rules leave t uncertain by up to their
// tolerances (a face hit is accepted at the first iterate whose residual is
// below 1e-4, so its t can be off by 1e-4 / |d.n|). A hit that passes the
// check takes a Newton step on the equations that define it, with the FP64
// residual just computed and the FP32 Jacobian at the hit:
//   face f:      x(xi) = o + t d, xi's fixed coordinate held (unknowns: the
//                two free coordinates and t), a 3x3 solve;
//   isosurface:  x(xi) = o + t d and u(xi) = iso (unknowns: xi and t), a
//                4x4 solve through J^-1.
// The step's error is quadratic in its size plus the FP32 Jacobian's
// relative error times its size, so a step of at most 1e-4 in t and xi
// (kPolishDone) lands within about 1e-8 times the equations' curvature and
// ends the polish; a larger step is followed by up to three more with the
// residual re-evaluated in FP64 (kPolishSteps). The hit keeps its
// element, face and kind; t, xi and u move to the root of the same equations,
// which leaves t within FP32 rounding of the exact root. A step in t larger
// than 2e-2 or in xi larger than 0.25, a non-finite one, or one that takes a
// face hit's free coordinates beyond 1.05 in magnitude (the reference
// accepts up to 1.001, and an accepted hit's exact root can lie a little
// further out) leaves the hit as the solver returned it.
#pragma once

#include <cuda_runtime.h>

#include "ho_device.cuh"
#include "ho_layout.h"

namespace ho {

// Tolerances of the check, FP64 and absolute (the scene is O(1)): the face
// acceptance 1e-4 and the isosurface criterion 1e-5, each with room for the
// FP32 rounding of the returned point.
constexpr double kCheckFaceTol = 1.5e-4;
constexpr double kCheckIsoPosTol = 1e-4;
constexpr double kCheckIsoFieldTol = 2e-5;

// Knuth's TwoSum: s + e == a + b exactly (round-to-nearest FP32; the
// intrinsics keep the compiler from fusing or reordering the steps).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// A double-single number: the unevaluated sum hi + lo of two floats, |lo| at
// most half an ulp of hi, about 48 significant bits.
struct Ds {
  float hi, lo;
};

__device__ __forceinline__ Ds ds_of(double x) {
  const float h = __double2float_rn(x);
  return {h, __double2float_rn(x - static_cast<double>(h))};
}

// (s, e) with s + e == a + b exactly, s the rounded sum (renormalisation).
__device__ __forceinline__ Ds ds_norm(float a, float b) {
  Ds r;
  two_sum(a, b, r.hi, r.lo);
  return r;
}

__device__ __forceinline__ Ds ds_add(Ds a, Ds b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  return ds_norm(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}

// The product's high part exact by an FMA-based TwoProduct, the cross terms
// added in FP32.
__device__ __forceinline__ Ds ds_mul(Ds a, Ds b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return ds_norm(p, e);
}

__device__ __forceinline__ Ds ds_sub(Ds a, Ds b) { return ds_add(a, {-b.hi, -b.lo}); }
// times a power of two (exact)
__device__ __forceinline__ Ds ds_scale2(Ds a, float s) { return {__fmul_rn(a.hi, s), __fmul_rn(a.lo, s)}; }

// Modified-A basis values in double-single, the recurrence of basis_val
// (the constants A_m, B_m rounded from FP64).
template <int N>
__device__ __forceinline__ void basis_val_ds(Ds x, Ds (&a)[N]) {
  const Ds one = {1.f, 0.f};
  a[0] = ds_scale2(ds_sub(one, x), 0.5f);
  if (N > 1) a[1] = ds_scale2(ds_add(one, x), 0.5f);
  const Ds w = ds_scale2(ds_sub(one, ds_mul(x, x)), 0.25f);
  Ds pm2 = one, pm1 = ds_scale2(x, 2.f);
#pragma unroll
  for (int i = 2; i < N; ++i) {
    const int m = i - 2;
    Ds p;
    if (m == 0) p = one;
    else if (m == 1) p = pm1;
    else {
      const Ds A = ds_of(double((2 * m + 1) * (m + 1)) / double(m * (m + 2)));
      const Ds B = ds_of(double(m + 1) / double(m + 2));
      p = ds_sub(ds_mul(ds_mul(A, x), pm1), ds_mul(B, pm2));
      pm2 = pm1;
      pm1 = p;
    }
    a[i] = ds_mul(w, p);
  }
}

// Value of one coefficient block (rows padded to row_stride(N), a multiple of
// 4 floats, so a row is RS/4 aligned float4 loads), FP64-accurate, computed
// in double-single arithmetic on the FP32 pipes.
//
// The coefficients are FP32. The innermost sums sum_i c_i a_i: a_i = ah_i +
// al_i (two floats), c_i ah_i = p + ep exactly (TwoProduct), the running sum
// kept as sh + sl with TwoSum, the small parts added in FP32. The sums over j
// and k multiply and add double-single numbers (ds_mul, ds_add). Each
// operation is good to about 2^-44 relative, below what the check and the
// polish need by orders of magnitude (the residuals agree with the FP64
// oracle's to 1e-10), and no FP64 instruction runs per coefficient or per
// row: GB300's FP64 rate is a small fraction of its FP32 rate, and with FP64
// sums over j and k the check kernel kept the FP64 pipe 72% busy.
template <int N>
__device__ double value64(const float* __restrict__ blk, const float (&ah)[N], const float (&al)[N],
                          const Ds (&as)[N], const Ds (&at)[N]) {
  constexpr int RS = row_stride(N);
  static_assert(RS % 4 == 0, "rows are whole float4s");
  Ds v = {0.f, 0.f};
#pragma unroll 1
  for (int k = 0; k < N; ++k) {
    Ds q = {0.f, 0.f};
#pragma unroll
    for (int j = 0; j < N; ++j) {
      const float4* row = reinterpret_cast<const float4*>(blk + (k * N + j) * RS);
      float c[RS];
#pragma unroll
      for (int i4 = 0; i4 < RS / 4; ++i4) {
        const float4 t4 = __ldg(row + i4);
        c[4 * i4] = t4.x;
        c[4 * i4 + 1] = t4.y;
        c[4 * i4 + 2] = t4.z;
        c[4 * i4 + 3] = t4.w;
      }
      float sh = 0.f, sl = 0.f;
#pragma unroll
      for (int i = 0; i < N; ++i) {
        const float p = __fmul_rn(c[i], ah[i]);
        const float ep = __fmaf_rn(c[i], ah[i], -p);
        float s, es;
        two_sum(sh, p, s, es);
        sh = s;
        sl = __fadd_rn(sl, __fadd_rn(__fadd_rn(es, ep), __fmul_rn(c[i], al[i])));
      }
      q = ds_add(q, ds_mul(ds_norm(sh, sl), as[j]));
    }
    Ds atk = at[0];  // at[k] by selection: the array stays in registers
#pragma unroll
    for (int kk = 1; kk < N; ++kk)
      if (kk == k) atk = at[kk];
    v = ds_add(v, ds_mul(q, atk));
  }
  return static_cast<double>(v.hi) + static_cast<double>(v.lo);
}

// The FP64 residual vector r = x(xi) - (o + t d) of a point in element elem,
// and the field value u(xi) (0 when unused).
template <int N>
__device__ __noinline__ void fp64_residual_vec(const float* __restrict__ rec_all, int elem, float3 o, float3 d,
                                               double t, double x0, double x1, double x2, bool want_field,
                                               double* __restrict__ r, double& u) {
  const float* rec = rec_all + static_cast<int64_t>(elem) * record_floats(N);
  Ds rd[N], sd[N], td[N];  // the basis values in r, s, t, double-single
  basis_val_ds<N>(ds_of(x0), rd);
  basis_val_ds<N>(ds_of(x1), sd);
  basis_val_ds<N>(ds_of(x2), td);
  float ah[N], al[N];  // the r values' two parts
#pragma unroll
  for (int i = 0; i < N; ++i) {
    ah[i] = rd[i].hi;
    al[i] = rd[i].lo;
  }
  r[0] = value64<N>(rec, ah, al, sd, td) - (static_cast<double>(o.x) + t * d.x);
  r[1] = value64<N>(rec + block_floats(N), ah, al, sd, td) - (static_cast<double>(o.y) + t * d.y);
  r[2] = value64<N>(rec + 2 * block_floats(N), ah, al, sd, td) - (static_cast<double>(o.z) + t * d.z);
  u = want_field ? value64<N>(rec + 3 * block_floats(N), ah, al, sd, td) : 0.0;
}

// The FP64 residuals of a hit at xi in element elem: the largest component
// of x(xi) - (o + t d), and the field value u(xi) (0 when unused).
template <int N>
__device__ void fp64_residuals(const float* __restrict__ rec_all, int elem, float3 o, float3 d, float t, float3 xi,
                               bool want_field, double& rpos, double& u) {
  double r[3];
  fp64_residual_vec<N>(rec_all, elem, o, d, t, xi.x, xi.y, xi.z, want_field, r, u);
  rpos = fmax(fabs(r[0]), fmax(fabs(r[1]), fabs(r[2])));
}

// Newton steps of the polish at most: the first uses the FP64 residual of the
// check; each later one re-evaluates it at the new point, and also the FP32
// Jacobian when the step before moved xi by more than 1e-3 (otherwise it
// keeps the previous one: a chord step, whose error shrinks by about the
// relative change of J across that step).
constexpr int kPolishSteps = 4;
// A step at most this large in t and in xi ends the polish without another
// FP64 evaluation (its remaining error is about its square), where the ray
// meets the surface at |cos| >= 0.2.
constexpr double kPolishDone = 1e-4;

// One Newton step on a hit's defining equations (file header): from the
// FP64 residual r and field value u at (t, xi), with the FP32 Jacobian J and
// xi-gradient g of the field at the hit. Returns false when the step is not
// usable (singular, too large, not finite).
__device__ __forceinline__ bool polish_step(const HitState& h, float3 d, float iso, const float (&J)[9], float3 g,
                                            const double (&r)[3], double u, double (&dx)[3], double& dt) {
  if (h.kind == HO_HIT_FACE) {
    int fixed, ua, va;
    float val;
    face_param(h.face, fixed, val, ua, va);
    // Cramer's rule on [J_u J_v -d] (du, dv, dt) = -r
    const double a0 = J[ua], a1 = J[3 + ua], a2 = J[6 + ua];
    const double b0 = J[va], b1 = J[3 + va], b2 = J[6 + va];
    const double c0 = -static_cast<double>(d.x), c1 = -static_cast<double>(d.y), c2 = -static_cast<double>(d.z);
    const double det = a0 * (b1 * c2 - b2 * c1) - b0 * (a1 * c2 - a2 * c1) + c0 * (a1 * b2 - a2 * b1);
    if (!(fabs(det) > 0.0)) return false;
    const double q0 = -r[0], q1 = -r[1], q2 = -r[2];
    const double du = (q0 * (b1 * c2 - b2 * c1) - b0 * (q1 * c2 - q2 * c1) + c0 * (q1 * b2 - q2 * b1)) / det;
    const double dv = (a0 * (q1 * c2 - q2 * c1) - q0 * (a1 * c2 - a2 * c1) + c0 * (a1 * q2 - a2 * q1)) / det;
    dt = (a0 * (b1 * q2 - b2 * q1) - b0 * (a1 * q2 - a2 * q1) + q0 * (a1 * b2 - a2 * b1)) / det;
    dx[0] = dx[1] = dx[2] = 0.0;
    dx[ua] = du;
    dx[va] = dv;
  } else {
    // J dxi - d dt = -r, g . dxi = -(u - iso): dxi = a + b dt with
    // a = -J^-1 r, b = J^-1 d
    const double j0 = J[0], j1 = J[1], j2 = J[2], j3 = J[3], j4 = J[4], j5 = J[5], j6 = J[6], j7 = J[7], j8 = J[8];
    const double k0 = j4 * j8 - j5 * j7, k1 = j2 * j7 - j1 * j8, k2 = j1 * j5 - j2 * j4;
    const double k3 = j5 * j6 - j3 * j8, k4 = j0 * j8 - j2 * j6, k5 = j2 * j3 - j0 * j5;
    const double k6 = j3 * j7 - j4 * j6, k7 = j1 * j6 - j0 * j7, k8 = j0 * j4 - j1 * j3;
    const double det = j0 * k0 + j1 * k3 + j2 * k6;
    if (!(fabs(det) > 0.0)) return false;
    const double id = 1.0 / det;
    const double a[3] = {-(k0 * r[0] + k1 * r[1] + k2 * r[2]) * id, -(k3 * r[0] + k4 * r[1] + k5 * r[2]) * id,
                         -(k6 * r[0] + k7 * r[1] + k8 * r[2]) * id};
    const double b[3] = {(k0 * d.x + k1 * d.y + k2 * d.z) * id, (k3 * d.x + k4 * d.y + k5 * d.z) * id,
                         (k6 * d.x + k7 * d.y + k8 * d.z) * id};
    const double gb = g.x * b[0] + g.y * b[1] + g.z * b[2];
    if (!(fabs(gb) > 0.0)) return false;
    dt = (-(u - static_cast<double>(iso)) - (g.x * a[0] + g.y * a[1] + g.z * a[2])) / gb;
    for (int k = 0; k < 3; ++k) dx[k] = a[k] + b[k] * dt;
  }
  // a face hit accepted at a residual of 1e-4 is up to about 1e-4 / |d.n|
  // off in t and that over |J| (about half the element size) in xi, which on
  // near-grazing rays reaches 1e-2 and 0.2: the limits leave room for that
  const double mx = fmax(fabs(dx[0]), fmax(fabs(dx[1]), fabs(dx[2])));
  return fabs(dt) <= 2e-2 && mx <= 0.25;  // also false for a NaN step
}

// The FP64 check of a hit (a miss always passes) and, when it passes, the
// polish (file header). Returns whether the hit passed; polished is set when
// the hit's t, xi and u were refined.
template <int N>
__device__ bool fp64_check_polish(const float* __restrict__ rec_all, const uint32_t* __restrict__ eflags, float3 o,
                                  float3 d, float iso, HitState& h, bool& polished, double* t64 = nullptr) {
  polished = false;
  if (t64) *t64 = h.t;
  if (h.kind == HO_HIT_MISS) return true;
  const bool iso_hit = h.kind != HO_HIT_FACE;
  const bool has_field = iso_hit || (__ldg(eflags + h.elem) & 1u) != 0;
  double r[3], u;
  fp64_residual_vec<N>(rec_all, h.elem, o, d, h.t, h.xi.x, h.xi.y, h.xi.z, has_field, r, u);
  const double rpos = fmax(fabs(r[0]), fmax(fabs(r[1]), fabs(r[2])));
  if (!iso_hit) {
    if (rpos > kCheckFaceTol) return false;
  } else if (rpos > kCheckIsoPosTol || fabs(u - static_cast<double>(iso)) > kCheckIsoFieldTol) {
    return false;
  }
  // FP32 Jacobian and field gradient at the hit
  const CoefRef<false> c{rec_all + static_cast<int64_t>(h.elem) * record_floats(N)};
  float J[9];
  float3 g = make_float3(0.f, 0.f, 0.f);
  auto jacobian_at = [&](float3 xi) {
    float xJ[12];
    geom_eval_raw<N, false>(c, xi, xJ);
    J[0] = xJ[1]; J[1] = xJ[2]; J[2] = xJ[3];
    J[3] = xJ[5]; J[4] = xJ[6]; J[5] = xJ[7];
    J[6] = xJ[9]; J[7] = xJ[10]; J[8] = xJ[11];
    if (has_field) {
      float ug[4];
      field_eval_raw<N, false>(c.at(3 * block_floats(N)), xi, ug);
      g = make_float3(ug[1], ug[2], ug[3]);
    }
  };
  jacobian_at(h.xi);
  const float dn = fabsf(h.n.x * d.x + h.n.y * d.y + h.n.z * d.z);
  const bool steep = dn >= 0.2f * sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
  double t = h.t, x0 = h.xi.x, x1 = h.xi.y, x2 = h.xi.z, un = u;
  for (int step = 0; step < kPolishSteps; ++step) {
    double dx[3], dt;
    if (!polish_step(h, d, iso, J, g, r, u, dx, dt)) return true;
    t += dt;
    x0 += dx[0];
    x1 += dx[1];
    x2 += dx[2];
    un = u + (g.x * dx[0] + g.y * dx[1] + g.z * dx[2]);
    // a step this small leaves an error far below FP32 rounding of t and xi;
    // on a ray that meets the surface at a shallow angle the equations are
    // ill-conditioned (the error grows like 1/|d.n|), so there only a step
    // below FP32 rounding ends the polish without another FP64 evaluation
    const double mx = fmax(fabs(dx[0]), fmax(fabs(dx[1]), fabs(dx[2])));
    const double done = steep ? kPolishDone : 1e-7;
    if (step + 1 == kPolishSteps || (mx <= done && fabs(dt) <= done)) break;
    if (mx > 1e-3)
      jacobian_at(make_float3(static_cast<float>(x0), static_cast<float>(x1), static_cast<float>(x2)));
    fp64_residual_vec<N>(rec_all, h.elem, o, d, t, x0, x1, x2, has_field, r, u);
    un = u;
  }
  if (h.kind == HO_HIT_FACE) {
    int fixed, ua, va;
    float val;
    face_param(h.face, fixed, val, ua, va);
    const double pu = ua == 0 ? x0 : (ua == 1 ? x1 : x2), pv = va == 0 ? x0 : (va == 1 ? x1 : x2);
    // the reference accepts a face hit up to 1.001 in its free coordinates;
    // the exact root of an accepted hit can lie a little further out
    if (!(fabs(pu) <= 1.05 && fabs(pv) <= 1.05)) return true;
  }
  h.t = static_cast<float>(t);
  h.xi = make_float3(static_cast<float>(x0), static_cast<float>(x1), static_cast<float>(x2));
  if (has_field) h.u = static_cast<float>(un);
  if (t64) *t64 = t;
  polished = true;
  return true;
}

// The FP64 tie rule between a ray's best hit (already checked and polished,
// exact root at t_best) and its tie partner: the partner is checked and
// polished the same way; if it passes, the nearer exact root wins, and where
// the two roots coincide within 1e-7 of t (one surface point: a shared face,
// an edge), the lower element index, then the lower face index. Returns true
// when the partner replaced the best hit (flags carried over); the answer
// carries HO_FLAG_TIE either way.
template <int N>
__device__ __noinline__ bool fp64_tie_rule(const float* __restrict__ rec_all, const uint32_t* __restrict__ eflags, float3 o,
                              float3 d, float iso, HitState& best, double t_best, HitState tie) {
  best.flags |= HO_FLAG_TIE;
  bool polished;
  double t_tie;
  if (!fp64_check_polish<N>(rec_all, eflags, o, d, iso, tie, polished, &t_tie)) return false;
  const double eps = 1e-7 * fmax(1.0, fabs(t_best));
  bool wins;
  if (t_tie < t_best - eps) wins = true;
  else if (t_tie > t_best + eps) wins = false;
  else wins = tie.elem < best.elem || (tie.elem == best.elem && tie.face < best.face);
  if (!wins) return false;
  tie.flags = best.flags;
  best = tie;
  return true;
}

}  // namespace ho
