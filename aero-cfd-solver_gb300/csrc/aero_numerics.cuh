// aero_numerics.cuh -- per-face and per-cell arithmetic of the 2D Euler path, written for
// the device (sm_103a) and templated on the bulk type T (float or double).
//
// The operation order and branch structure follow the reference functions cited per
// function (paths relative to the AeroCFD project root) so that, apart from FMA
// contraction, the device produces the reference's numbers. In 2D the reference carries
// a fifth component (rho*w, w) that is identically zero: every term it contributes is an
// exact +0, so the device works on four components (rho, rho*u, rho*v, rho*E) /
// (rho, u, v, p) and writes 0 for the fifth.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include <type_traits>

namespace aero {

template <class T>
struct Kn {
  static constexpr T rho_floor = T(1.0e-8);
  static constexpr T p_floor = T(1.0e-8);
  static constexpr T wave_floor = T(1.0e-8);
  static constexpr T low_mach_min = T(1.0e-4);
  static constexpr T all_speed_floor = T(1.0e-6);
  static constexpr T smooth_eps = T(1.0e-6);
  static constexpr T vol_floor = T(1.0e-12);
};

// Double compares on the device run on the integer pipe. GB300 executes double-precision
// compares (and max / min) on the same narrow FP64 pipe as its double arithmetic, and the
// FP64 face pass keeps that pipe busy. A double's bit pattern with the magnitude bits of a
// negative value inverted (its orderable key) orders like the value, so the integer pipe can
// compare instead. dlt equals a < b for every pair of non-NaN doubles, the two zeros
// included. A NaN operand, which only a non-finite state produces, orders by its bit pattern:
// above +inf with the sign bit clear, below -inf with it set.
__device__ __forceinline__ long long dkey(double x) {
  const long long b = __double_as_longlong(x);
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ bool dlt(double a, double b) {
  const long long both = __double_as_longlong(a) | __double_as_longlong(b);
  return dkey(a) < dkey(b) && (both & 0x7fffffffffffffffLL) != 0;  // -0 < +0 is false
}
// a < b in the numerics' kernels: dlt for two doubles on the device, the operator otherwise
template <class A, class B>
__host__ __device__ __forceinline__ bool slt(A a, B b) {
  return a < b;
}
__host__ __device__ __forceinline__ bool slt(double a, double b) {
#ifdef __CUDA_ARCH__
  return dlt(a, b);
#else
  return a < b;
#endif
}

// std::max / std::min / std::clamp semantics (NaN handling included).
template <class T>
__host__ __device__ __forceinline__ T smax(T a, T b) {
  return (a < b) ? b : a;
}
template <class T>
__host__ __device__ __forceinline__ T smin(T a, T b) {
  return (b < a) ? b : a;
}
template <class T>
__host__ __device__ __forceinline__ T sclamp(T v, T lo, T hi) {
  return (v < lo) ? lo : ((hi < v) ? hi : v);
}
// Float on the device: the hardware's NaN-propagating max / min (one instruction where the
// forms above take a compare and a select). Equal to them for every pair of numbers, up to
// the sign of a zero result; a NaN in either operand gives NaN, where std::max(a, NaN) gives
// a. A NaN operand only arises from a non-finite state, which the non-finite trap stops
// either way. sclamp is max-then-min, equal to the form above whenever lo <= hi (every use).
template <>
__host__ __device__ __forceinline__ float smax<float>(float a, float b) {
#ifdef __CUDA_ARCH__
  float r;
  asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
#else
  return (a < b) ? b : a;
#endif
}
template <>
__host__ __device__ __forceinline__ float smin<float>(float a, float b) {
#ifdef __CUDA_ARCH__
  float r;
  asm("min.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
#else
  return (b < a) ? b : a;
#endif
}
template <>
__host__ __device__ __forceinline__ float sclamp<float>(float v, float lo, float hi) {
  return smin<float>(smax<float>(v, lo), hi);
}
// Double on the device: the same selections with the compares on the integer pipe (slt);
// equal to the forms above for every pair of non-NaN values, a NaN operand ordering as in dlt.
template <>
__host__ __device__ __forceinline__ double smax<double>(double a, double b) {
  return slt(a, b) ? b : a;
}
template <>
__host__ __device__ __forceinline__ double smin<double>(double a, double b) {
  return slt(b, a) ? b : a;
}
template <>
__host__ __device__ __forceinline__ double sclamp<double>(double v, double lo, double hi) {
  return slt(v, lo) ? lo : (slt(hi, v) ? hi : v);
}
// Quotient a / b. Float on the device: the approximate divide (__fdividef, 2 ulp for divisors
// of magnitude 2^-126 to 2^126, the range of every divisor here: floored densities, pressures,
// sound speeds and wave-speed differences). The float division as this library compiles it
// (also 2 ulp) adds full-range scaling: on the solver's inputs both give the same quotients
// (a 524k-cell low-Mach run is bit-identical), and this one issues fewer instructions.
template <class T>
__host__ __device__ __forceinline__ T sdiv(T a, T b) {
  return a / b;
}
template <>
__host__ __device__ __forceinline__ float sdiv<float>(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fdividef(a, b);
#else
  return a / b;
#endif
}
template <class T>
__host__ __device__ __forceinline__ T sabs(T x) {
  return fabs(x);
}
template <>
__host__ __device__ __forceinline__ float sabs<float>(float x) {
  return fabsf(x);
}
// double on the device: the sign bit cleared on the integer pipe (fabs, bit for bit)
template <>
__host__ __device__ __forceinline__ double sabs<double>(double x) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(__double_as_longlong(x) & 0x7fffffffffffffffLL);
#else
  return fabs(x);
#endif
}
template <class T>
__host__ __device__ __forceinline__ T ssqrt(T x) {
  return sqrt(x);
}
template <>
__host__ __device__ __forceinline__ float ssqrt<float>(float x) {
  return sqrtf(x);
}
template <class T>
__host__ __device__ __forceinline__ bool sfinite(T x) {
  return isfinite(x);
}
// float: |x| < inf is false exactly for the infinities and NaN (one compare)
template <>
__host__ __device__ __forceinline__ bool sfinite<float>(float x) {
  return fabsf(x) < INFINITY;
}
// double on the device: the exponent field is all ones exactly for the infinities and NaN
template <>
__host__ __device__ __forceinline__ bool sfinite<double>(double x) {
#ifdef __CUDA_ARCH__
  return ((__double_as_longlong(x) >> 52) & 0x7ff) != 0x7ff;
#else
  return isfinite(x);
#endif
}

template <class T>
struct Prim {
  T r, u, v, p;
};
template <class T>
struct Cons {
  T r, ru, rv, rE;
};
template <class T>
struct Flux {
  T m, fx, fy, e;
};

// euler_flux.cpp:101-113
template <class T>
__device__ __forceinline__ Cons<T> prim_to_cons(const Prim<T>& w, T gamma) {
  Cons<T> c;
  c.r = smax(w.r, Kn<T>::rho_floor);
  c.ru = c.r * w.u;
  c.rv = c.r * w.v;
  const T ke = T(0.5) * c.r * (w.u * w.u + w.v * w.v);
  const T p = smax(w.p, Kn<T>::p_floor);
  c.rE = sdiv(p, gamma - T(1)) + ke;
  return c;
}

// euler_flux.cpp:115-127 from the floored density r and its reciprocal inv
template <class T>
__device__ __forceinline__ Prim<T> cons_to_prim_from(const Cons<T>& c, T gamma, T r, T inv) {
  Prim<T> w;
  w.r = r;
  w.u = c.ru * inv;
  w.v = c.rv * inv;
  const T ke = T(0.5) * w.r * (w.u * w.u + w.v * w.v);
  w.p = smax((gamma - T(1)) * (c.rE - ke), Kn<T>::p_floor);
  return w;
}
// euler_flux.cpp:115-127. *inv_out, when given, receives the 1/rho the velocities use.
template <class T>
__device__ __forceinline__ Prim<T> cons_to_prim(const Cons<T>& c, T gamma, T* inv_out = nullptr) {
  const T r = smax(c.r, Kn<T>::rho_floor);
  const T inv = sdiv(T(1), r);
  if (inv_out) *inv_out = inv;
  return cons_to_prim_from(c, gamma, r, inv);
}

// euler_flux.cpp:129-144 with the energy floor pf = p_floor / (gamma - 1) given; returns the
// 1/rho of the result (rho is floored and not changed after it), which is the reciprocal
// cons_to_prim of the result forms
template <class T>
__device__ __forceinline__ T enforce_physical_pf(Cons<T>* s, T gamma, T pf) {
  s->r = smax(s->r, Kn<T>::rho_floor);
  const T inv = sdiv(T(1), s->r);
  const T u = s->ru * inv, v = s->rv * inv;
  const T ke = T(0.5) * s->r * (u * u + v * v);
  s->rE = smax(s->rE, ke + pf);
  const T p = (gamma - T(1)) * (s->rE - ke);
  if (slt(p, Kn<T>::p_floor)) s->rE = ke + pf;
  return inv;
}
// euler_flux.cpp:129-144
template <class T>
__device__ __forceinline__ void enforce_physical(Cons<T>* s, T gamma) {
  enforce_physical_pf(s, gamma, sdiv(Kn<T>::p_floor, gamma - T(1)));
}

// euler_flux.cpp:150-152
template <class T>
__device__ __forceinline__ T sound_speed(const Prim<T>& w, T gamma) {
  return ssqrt(smax(sdiv(gamma * w.p, smax(w.r, Kn<T>::rho_floor)), T(0)));
}

// Double precision spends a division on the FP64 pipe, which GB300 runs at a small fraction
// of the float rate. Where a state's 1/rho is already formed, the FP64 face pass multiplies
// by it instead of dividing by rho again. The product is within an ulp of the quotient,
// far inside the FP64 path's 1e-12 agreement with the FP64 oracle. Float and dual numbers
// keep the quotient.
template <class T>
constexpr bool kReuseInverse = std::is_same<T, double>::value;

// sound_speed of a state from cons_to_prim (w.r floored), given its 1/rho
template <class T>
__device__ __forceinline__ T sound_speed_inv(const Prim<T>& w, T inv, T gamma) {
  if constexpr (kReuseInverse<T>) {
    return ssqrt(smax(gamma * w.p * inv, T(0)));
  } else {
    return sound_speed(w, gamma);
  }
}

template <class T>
__device__ __forceinline__ T vmag(const Prim<T>& w) {
  return ssqrt(w.u * w.u + w.v * w.v);
}

// preconditioning.cpp:17-22
template <class T>
__device__ __forceinline__ T local_mach(const Prim<T>& w, T gamma) {
  return sdiv(vmag(w), smax(sound_speed(w, gamma), Kn<T>::wave_floor));
}

// euler_flux.cpp:28-39
template <class T>
__device__ __forceinline__ Flux<T> physical_flux(const Cons<T>& c, const Prim<T>& w, T nx, T ny) {
  const T un = w.u * nx + w.v * ny;
  return {c.r * un, c.ru * un + nx * w.p, c.rv * un + ny * w.p, (c.rE + w.p) * un};
}

// euler_flux.cpp:45-51
template <class T>
__device__ __forceinline__ T with_sign_floor(T x) {
  if (!slt(sabs(x), Kn<T>::wave_floor)) return x;
  return !slt(x, T(0)) ? Kn<T>::wave_floor : -Kn<T>::wave_floor;
}

template <class T>
struct Speeds {
  T lm, lp, sr;
};

// euler_flux.cpp:58-74; the radius is also boundary_conditions.cpp:14-25.
template <class T>
__device__ __forceinline__ Speeds<T> precond_speeds(T un, T a, T acoustic_scale) {
  const T beta = sclamp(acoustic_scale, Kn<T>::low_mach_min, T(1));
  const T b2 = beta * beta;
  const T omb2 = T(1) - b2;
  const T ut = T(0.5) * (T(1) + b2) * un;
  const T disc = omb2 * omb2 * un * un + T(4) * b2 * a * a;
  const T ct = T(0.5) * ssqrt(smax(disc, T(0)));
  Speeds<T> s;
  s.lm = ut - ct;
  s.lp = ut + ct;
  // std::max({|un|, |lm|, |lp|, floor}) keeps the first of equal maxima
  T m = sabs(un);
  m = smax(m, sabs(s.lm));
  m = smax(m, sabs(s.lp));
  s.sr = smax(m, Kn<T>::wave_floor);
  return s;
}

// precond_speeds at acoustic scale 1 (no low-Mach scaling): beta = 1, so ut = un exactly and
// ct = sqrt(4 a^2) / 2 = a exactly in the reference's arithmetic (the correctly rounded square
// root of a rounded square returns the operand, and scaling by 4 is exact), and the largest of
// |un|, |un - a|, |un + a| (a >= 0) is the rounded |un| + a.
template <class T>
__device__ __forceinline__ Speeds<T> unit_speeds(T un, T a) {
  Speeds<T> s;
  s.lm = un - a;
  s.lp = un + a;
  s.sr = smax(sabs(un) + a, Kn<T>::wave_floor);
  return s;
}
// the speeds at the face's acoustic scale: LM false means the scale is exactly 1
template <class T, bool LM>
__device__ __forceinline__ Speeds<T> face_speeds(T un, T a, T as) {
  if constexpr (LM) {
    return precond_speeds(un, a, as);
  } else {
    return unit_speeds(un, a);
  }
}

// Settings of one residual evaluation that do not change within a launch
// (residual_assembly.hpp:12-31, preconditioning.hpp:9-15).
// 16-byte aligned, so that a kernel loads the fields it uses in vector loads.
template <class T>
struct alignas(16) FaceParams {
  Cons<T> farfield;
  T gamma;
  int limiter;  // 0 minmod, 1 venkat
  int precond;
  int low_mach_fix;
  int precond_farfield_bc;
  int as_fix;
  T mach_cutoff;
  T pc_mach_ref, pc_mach_min, pc_beta_min, pc_beta_max;
  T stab_floor;
  T as_cutoff, as_fmin, as_ramp;
  T inv_gm1;  // 1 / (gamma - 1), formed once per case (used by the FP64 face pass)
};

// prim_to_cons (euler_flux.cpp:101-113) in the face pass: in FP64 the energy's pressure term
// is p * (1 / (gamma - 1)) with the case's reciprocal (kReuseInverse)
template <class T>
__device__ __forceinline__ Cons<T> prim_to_cons_face(const Prim<T>& w, const FaceParams<T>& fp) {
  if constexpr (kReuseInverse<T>) {
    Cons<T> c;
    c.r = smax(w.r, Kn<T>::rho_floor);
    c.ru = c.r * w.u;
    c.rv = c.r * w.v;
    const T ke = T(0.5) * c.r * (w.u * w.u + w.v * w.v);
    const T p = smax(w.p, Kn<T>::p_floor);
    c.rE = p * fp.inv_gm1 + ke;
    return c;
  } else {
    return prim_to_cons(w, fp.gamma);
  }
}

// The two sides of a face in primitive form with the quantities the acoustic scale, the
// all-speed pressure scale and the flux all use, formed once per face: the reference's helpers
// each convert and derive them again from the conservative states by the same formulas (the
// values agree up to where the compiler contracts a multiply-add).
template <class T>
struct FaceSides {
  Prim<T> pl, pr;
  T unl, unr;  // normal velocities
  T al, ar;    // sound speeds
  T il, ir;    // 1/rho of each side
};
template <class T>
__device__ __forceinline__ FaceSides<T> face_sides(const Cons<T>& l, const Cons<T>& r, T nx, T ny, T gamma) {
  FaceSides<T> f;
  f.pl = cons_to_prim(l, gamma, &f.il);
  f.pr = cons_to_prim(r, gamma, &f.ir);
  f.unl = f.pl.u * nx + f.pl.v * ny;
  f.unr = f.pr.u * nx + f.pr.v * ny;
  f.al = sound_speed_inv(f.pl, f.il, gamma);
  f.ar = sound_speed_inv(f.pr, f.ir, gamma);
  return f;
}
// local Mach numbers |u| / max(a, floor) of both sides (preconditioning.cpp:17-22, the
// euler_flux.cpp:159-163 and :189-191 forms are the same expression)
template <class T>
struct SideMach {
  T al, ar;  // max(a, floor)
  T ml, mr;
};
template <class T>
__device__ __forceinline__ SideMach<T> side_mach(const FaceSides<T>& f) {
  SideMach<T> m;
  m.al = smax(f.al, Kn<T>::wave_floor);
  m.ar = smax(f.ar, Kn<T>::wave_floor);
  m.ml = sdiv(vmag(f.pl), m.al);
  m.mr = sdiv(vmag(f.pr), m.ar);
  return m;
}

// euler_flux.cpp:154-175 (prims already converted by the caller)
template <class T>
__device__ __forceinline__ T low_mach_dissipation_scale(const SideMach<T>& sm, T cutoff, T mach_ref) {
  if (cutoff <= T(0)) return T(1);
  const T fm = T(0.5) * (sm.ml + sm.mr);
  const T mstar = smax(fm, smax(mach_ref, Kn<T>::wave_floor));
  const T ratio = sdiv(mstar, smax(cutoff, Kn<T>::wave_floor));
  return sclamp(ratio, Kn<T>::low_mach_min, T(1));
}

// euler_flux.cpp:81-98 + 177-201
template <class T>
__device__ __forceinline__ T all_speed_pressure_scale(const FaceSides<T>& f, const SideMach<T>& sm,
                                                      const FaceParams<T>& fp) {
  const T mach = smax(T(0.5) * (sm.ml + sm.mr), Kn<T>::all_speed_floor);
  T mn = smax(T(0.5) * (sdiv(sabs(f.unl), sm.al) + sdiv(sabs(f.unr), sm.ar)), Kn<T>::all_speed_floor);
  mn = smin(mn, mach);
  mn = smax(mn, Kn<T>::all_speed_floor);
  const T cut = smax(fp.as_cutoff, Kn<T>::all_speed_floor);
  const T tfloor = sclamp(fp.as_fmin, Kn<T>::all_speed_floor, T(1));
  const T tn = sclamp(sdiv(mn, cut), tfloor, T(1));
  const T ratio = sclamp(sdiv(mach, cut), T(0), T(1));
  const T gate = ratio * ratio;
  const T tc = (T(1) - gate) * tn + gate;
  const T w = sclamp(fp.as_ramp, T(0), T(1));
  const T te = (T(1) - w) + w * tc;
  return sclamp(te, tfloor, T(1));
}

// euler_flux.cpp:203-239. ul/ur conservative, f their primitive sides.
template <class T, bool LM>
__device__ __forceinline__ Flux<T> rusanov(const Cons<T>& ul, const Cons<T>& ur, const FaceSides<T>& f, T nx,
                                           T ny, T as, T* mws) {
  const T unl = f.unl, unr = f.unr, al = f.al, ar = f.ar;
  const Prim<T>& pl = f.pl;
  const Prim<T>& pr = f.pr;
  const T smax_phys = smax(sabs(unl) + al, sabs(unr) + ar);
  const T sdiss = smax(face_speeds<T, LM>(unl, al, as).sr, face_speeds<T, LM>(unr, ar, as).sr);
  *mws = smax(smax_phys, Kn<T>::wave_floor);
  const Flux<T> fl = physical_flux(ul, pl, nx, ny), fr = physical_flux(ur, pr, nx, ny);
  const T hs = T(0.5) * sdiss;
  return {T(0.5) * (fl.m + fr.m) - hs * (ur.r - ul.r), T(0.5) * (fl.fx + fr.fx) - hs * (ur.ru - ul.ru),
          T(0.5) * (fl.fy + fr.fy) - hs * (ur.rv - ul.rv), T(0.5) * (fl.e + fr.e) - hs * (ur.rE - ul.rE)};
}

template <class T>
__device__ __forceinline__ bool finite4(T a, T b, T c, T d) {
  return sfinite(a) && sfinite(b) && sfinite(c) && sfinite(d);
}

// euler_flux.cpp:241-364. LM selects the all-speed pressure correction; with LM false the
// pressure scale is the constant 1 the reference uses when the fix is off.
template <class T, bool LM>
__device__ __forceinline__ Flux<T> hllc(const Cons<T>& ul, const Cons<T>& ur, const FaceSides<T>& f,
                                        const SideMach<T>& sm, T nx, T ny, const FaceParams<T>& fp, T as,
                                        T* mws, bool* fallback) {
  const Prim<T>& pl = f.pl;
  const Prim<T>& pr = f.pr;
  const T unl = f.unl, unr = f.unr, al = f.al, ar = f.ar;
  T ps = T(1);
  if (LM) {
    if (fp.as_fix) ps = all_speed_pressure_scale(f, sm, fp);
  }
  const T pavg = T(0.5) * (pl.p + pr.p);
  const T plc = pavg + ps * (pl.p - pavg);
  const T prc = pavg + ps * (pr.p - pavg);
  const Speeds<T> spl = face_speeds<T, LM>(unl, al, as);
  const Speeds<T> spr = face_speeds<T, LM>(unr, ar, as);
  const T s_l = smin(spl.lm, spr.lm);
  const T s_r = smax(spl.lp, spr.lp);
  const T slp = smin(unl - al, unr - ar);
  const T srp = smax(unl + al, unr + ar);
  *mws = smax(smax(sabs(slp), sabs(srp)), Kn<T>::wave_floor);
  *fallback = false;

  bool diffusive = slt(sabs(s_r - s_l), Kn<T>::wave_floor);
  Flux<T> fx;
  if (!diffusive) {
    const Flux<T> fl = physical_flux(ul, pl, nx, ny);
    const Flux<T> fr = physical_flux(ur, pr, nx, ny);
    if (!slt(s_l, T(0))) return fl;
    if (!slt(T(0), s_r)) return fr;
    const T rl = smax(pl.r, Kn<T>::rho_floor);
    const T rr = smax(pr.r, Kn<T>::rho_floor);
    const T denom = rl * (s_l - unl) - rr * (s_r - unr);
    diffusive = slt(sabs(denom), Kn<T>::wave_floor);
    if (!diffusive) {
      const T s_m = sdiv(prc - plc + rl * unl * (s_l - unl) - rr * unr * (s_r - unr), denom);
      // star states (euler_flux.cpp:313-334) on the side the contact selects; the other
      // side only enters the finiteness/positivity test, so both are formed.
      Cons<T> stl = ul, str = ur;
      {
        const T skun = s_l - unl, sksm = s_l - s_m;
        if (!(slt(sabs(skun), Kn<T>::wave_floor) || slt(sabs(sksm), Kn<T>::wave_floor))) {
          const T rs = sdiv(rl * skun, sksm);
          const T sh = s_m - unl;
          stl.r = rs;
          stl.ru = rs * (pl.u + sh * nx);
          stl.rv = rs * (pl.v + sh * ny);
          // rl is pl.r (cons_to_prim floors it), whose reciprocal the face sides hold
          const T et = kReuseInverse<T> ? ul.rE * f.il : sdiv(ul.rE, rl);
          const T pt = sdiv(plc, with_sign_floor(rl * skun));
          stl.rE = rs * (et + sh * (s_m + pt));
        }
      }
      {
        const T skun = s_r - unr, sksm = s_r - s_m;
        if (!(slt(sabs(skun), Kn<T>::wave_floor) || slt(sabs(sksm), Kn<T>::wave_floor))) {
          const T rs = sdiv(rr * skun, sksm);
          const T sh = s_m - unr;
          str.r = rs;
          str.ru = rs * (pr.u + sh * nx);
          str.rv = rs * (pr.v + sh * ny);
          const T et = kReuseInverse<T> ? ur.rE * f.ir : sdiv(ur.rE, rr);
          const T pt = sdiv(prc, with_sign_floor(rr * skun));
          str.rE = rs * (et + sh * (s_m + pt));
        }
      }
      // the w component of both star states is rho_star*(0 + shift*0), always finite
      diffusive = !finite4(stl.r, stl.ru, stl.rv, stl.rE) || !finite4(str.r, str.ru, str.rv, str.rE) ||
                  !slt(T(0), stl.r) || !slt(T(0), str.r);
      if (!diffusive) {
        if (!slt(s_m, T(0))) {
          fx = {fl.m + s_l * (stl.r - ul.r), fl.fx + s_l * (stl.ru - ul.ru), fl.fy + s_l * (stl.rv - ul.rv),
               fl.e + s_l * (stl.rE - ul.rE)};
        } else {
          fx = {fr.m + s_r * (str.r - ur.r), fr.fx + s_r * (str.ru - ur.ru), fr.fy + s_r * (str.rv - ur.rv),
               fr.e + s_r * (str.rE - ur.rE)};
        }
        diffusive = !finite4(fx.m, fx.fx, fx.fy, fx.e);
      }
    }
  }
  if (diffusive) {
    *fallback = true;
    fx = rusanov<T, LM>(ul, ur, f, nx, ny, as, mws);
  }
  return fx;
}

// preconditioning.cpp:9-15 + 24-32 on a primitive state
template <class T>
__device__ __forceinline__ T cell_beta(const Prim<T>& w, const FaceParams<T>& fp) {
  const T m = local_mach(w, fp.gamma);
  T target = m;
  target = smax(target, fp.pc_mach_ref);
  target = smax(target, fp.pc_mach_min);
  target = smax(target, Kn<T>::wave_floor);
  const T bmin = smax(fp.pc_beta_min, Kn<T>::low_mach_min);
  const T bmax = smax(bmin, fp.pc_beta_max);
  return sclamp(target, bmin, bmax);
}

// residual_assembly.cpp:16-20
template <class T>
__device__ __forceinline__ T smooth_max(T a, T b) {
  const T d = a - b;
  return T(0.5) * (a + b + ssqrt(d * d + Kn<T>::smooth_eps * Kn<T>::smooth_eps));
}

// preconditioning.cpp:34-49 (face beta) and residual_assembly.cpp:31-51 (acoustic scale),
// from the two conservative face states. Without LM the scale is exactly 1.
template <class T, bool LM>
__device__ __forceinline__ T face_acoustic_scale(const FaceSides<T>& f, const SideMach<T>& sm,
                                                 const FaceParams<T>& fp) {
  if (!LM) return T(1);
  const Prim<T>& pl = f.pl;
  const Prim<T>& pr = f.pr;
  T s = T(1);
  if (fp.precond) {
    const Prim<T> avg{T(0.5) * (pl.r + pr.r), T(0.5) * (pl.u + pr.u), T(0.5) * (pl.v + pr.v),
                      T(0.5) * (pl.p + pr.p)};
    s = sclamp(cell_beta(avg, fp), Kn<T>::low_mach_min, T(1));
  }
  if (fp.low_mach_fix) s = smin(s, low_mach_dissipation_scale(sm, fp.mach_cutoff, fp.pc_mach_ref));
  s = sclamp(s, Kn<T>::low_mach_min, T(1));
  const T fm = T(0.5) * (sm.ml + sm.mr);
  const T fl = sclamp(fp.stab_floor, T(0), T(1));
  const T stab = sclamp(smooth_max(fm, fl), Kn<T>::low_mach_min, T(1));
  return smax(s, stab);
}

// boundary_conditions.cpp:27-78
template <class T>
__device__ __forceinline__ Cons<T> precond_farfield_state(const Cons<T>& in, T nx, T ny,
                                                          const FaceParams<T>& fp, T as) {
  const T gamma = fp.gamma;
  const Prim<T> pi = cons_to_prim(in, gamma), pf = cons_to_prim(fp.farfield, gamma);
  const T uni = pi.u * nx + pi.v * ny, unf = pf.u * nx + pf.v * ny;
  const T ai = smax(sound_speed(pi, gamma), Kn<T>::rho_floor);
  const T af = smax(sound_speed(pf, gamma), Kn<T>::rho_floor);
  const T rho_ref = smax(T(0.5) * (pi.r + pf.r), Kn<T>::rho_floor);
  const T a_ref = smax(T(0.5) * (ai + af), Kn<T>::rho_floor);
  const T a_t = smax(sclamp(as, Kn<T>::low_mach_min, T(1)) * a_ref, Kn<T>::all_speed_floor);
  if (sabs(uni) >= a_t) return (uni >= T(0)) ? in : fp.farfield;
  const T rp = uni + sdiv(pi.p, rho_ref * a_t);
  const T rm = unf - sdiv(pf.p, rho_ref * a_t);
  const T unb = T(0.5) * (rp + rm);
  const T pb = smax(T(0.5) * rho_ref * a_t * (rp - rm), Kn<T>::rho_floor);
  const bool inflow = unb < T(0);
  const T tu = inflow ? (pf.u - unf * nx) : (pi.u - uni * nx);
  const T tv = inflow ? (pf.v - unf * ny) : (pi.v - uni * ny);
  const T rb = inflow ? pf.r : pi.r;
  const T pb0 = inflow ? pf.p : pi.p;
  const T ab = inflow ? af : ai;
  Prim<T> b;
  b.r = smax(rb + sdiv(pb - pb0, smax(ab * ab, Kn<T>::rho_floor)), Kn<T>::rho_floor);
  b.u = unb * nx + tu;
  b.v = unb * ny + tv;
  b.p = pb;
  return prim_to_cons_face(b, fp);
}

// euler_flux.cpp:366-395
template <class T, int FLUX, bool LM>
__device__ __forceinline__ Flux<T> face_flux(const Cons<T>& l, const Cons<T>& r, const FaceSides<T>& f,
                                             const SideMach<T>& sm, T nx, T ny, const FaceParams<T>& fp, T as,
                                             T* mws, bool* fallback) {
  if (FLUX == 1) return hllc<T, LM>(l, r, f, sm, nx, ny, fp, as, mws, fallback);
  *fallback = false;
  return rusanov<T, LM>(l, r, f, nx, ny, as, mws);
}

// reconstruction.cpp:121-146
template <class T>
__device__ __forceinline__ T limit(int lim, T a, T b) {
  if (!slt(T(0), a * b)) return T(0);  // a * b <= 0 (compares through slt)
  if (lim == 1) {
    const T eps2 = T(1.0e-12) * (T(1) + a * a + b * b);
    const T num = (b * b + T(2) * a * b + eps2) * a;
    const T den = a * a + T(2) * b * b + a * b + eps2;
    if (!slt(T(1.0e-20), sabs(den))) return T(0);
    const T x = sdiv(num, den);
    if (!sfinite(x)) return T(0);
    if (slt(T(0), a)) return sclamp(x, T(0), a);
    return sclamp(x, a, T(0));
  }
  return slt(sabs(a), sabs(b)) ? a : b;
}

// residual_assembly.cpp:53-58 (w is 0, always finite)
template <class T>
__device__ __forceinline__ bool valid_prim(const Prim<T>& w) {
  return sfinite(w.r) && sfinite(w.u) && sfinite(w.v) && sfinite(w.p) && slt(Kn<T>::rho_floor, w.r) &&
         slt(Kn<T>::p_floor, w.p);
}

}  // namespace aero
