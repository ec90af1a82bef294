// Arithmetic policies for one lifting update
//   g[k] = c0 * g[k - s] + c1 * g[k] + c2 * g[k + s]
// (paliwa/paliwa_transform.hpp:46-49). Every policy keeps the reference's
// evaluation order ((c0*lo + c1*me) + c2*up).
#pragma once

#include <cuda_runtime.h>

namespace pgb {

// One lifting pass's coefficients in both precisions, converted once on the
// host: on GB300 a double->float conversion runs on the (slow) FP64 pipe, so
// none may happen per update.
struct Coeffs {
  double c0, c1, c2;
  float f0, f1, f2;
};

// ---------------------------------------------------------------------------
// Plain IEEE arithmetic in T (double or float).
//
// ExactProducts: the host has checked that every coefficient is 0 or a power
// of two, so each product c*x is exact. Then
//   fma(c0, lo, c1*me) == round(round(c0*lo) + round(c1*me))
// and the fused form is bit-identical to the reference's separately rounded
// expression while issuing two FMAs per update (one more multiply only when
// c1 != 1). Otherwise every product and sum is rounded separately with the
// _rn intrinsics, which the compiler never contracts.
template <typename T, bool ExactProducts> struct Plain {
  using V = T;
  using Store = T;
  static __device__ __forceinline__ V load(Store x) { return x; }
  static __device__ __forceinline__ Store store(V x) { return x; }

  static constexpr bool kPacked = false;

  // C1: the middle coefficient is exactly 1 (skips one multiply).
  static __device__ __forceinline__ T k0(Coeffs const &c) {
    if constexpr (sizeof(T) == 8) return c.c0; else return c.f0;
  }
  static __device__ __forceinline__ T k1(Coeffs const &c) {
    if constexpr (sizeof(T) == 8) return c.c1; else return c.f1;
  }
  static __device__ __forceinline__ T k2(Coeffs const &c) {
    if constexpr (sizeof(T) == 8) return c.c2; else return c.f2;
  }

  template <bool C1>
  static __device__ __forceinline__ V update(Coeffs const &c, V lo, V me,
                                             V up) {
    if constexpr (ExactProducts) {
      V t = C1 ? me : mul(k1(c), me);
      t = fma(k0(c), lo, t);
      return fma(k2(c), up, t);
    } else {
      V t = add(mul(k0(c), lo), C1 ? me : mul(k1(c), me));
      return add(t, mul(k2(c), up));
    }
  }

 private:
  static __device__ __forceinline__ double mul(double a, double b) {
    return __dmul_rn(a, b);
  }
  static __device__ __forceinline__ float mul(float a, float b) {
    return __fmul_rn(a, b);
  }
  static __device__ __forceinline__ double add(double a, double b) {
    return __dadd_rn(a, b);
  }
  static __device__ __forceinline__ float add(float a, float b) {
    return __fadd_rn(a, b);
  }
  static __device__ __forceinline__ double fma(double a, double b, double c) {
    return __fma_rn(a, b, c);
  }
  static __device__ __forceinline__ float fma(float a, float b, float c) {
    return __fmaf_rn(a, b, c);
  }
};

// ---------------------------------------------------------------------------
// FP32 storage with compensated (double-float) arithmetic.
//
// A value in registers is an unevaluated pair h + l of floats. Loads start
// with l = 0. Each update evaluates c0*lo + c1*me + c2*up with error-free
// transformations (FMA-based TwoProd, Knuth TwoSum), so rounding errors do not
// accumulate along the level chain; the pair is rounded to one float only
// when it is stored, i.e. once per dimension. Every level runs in this
// arithmetic, the coarsest included: its 48-bit significand is far below
// the float storage that every value is rounded to, so FP64 steps would not
// change what is stored (the mass-conservation tests hold the FP32c result
// to the storage-rounding bound).
struct DF {
  float h, l;
};

__device__ __forceinline__ DF two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ DF fast_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return {s, e};
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
  DF s = two_sum(a.h, b.h);
  float e = __fadd_rn(s.l, __fadd_rn(a.l, b.l));
  return fast_two_sum(s.h, e);
}
// c * a for a float coefficient c: TwoProd on the high part plus the low part.
__device__ __forceinline__ DF df_scale(float c, DF a) {
  float p = __fmul_rn(c, a.h);
  float e = __fmaf_rn(c, a.h, -p);
  e = __fmaf_rn(c, a.l, e);
  return {p, e};
}

// Sym: every pass of the launch has c0 == c2 and only exact-scaler
// coefficients (true for all of paliwa's wavelet tables). The update is then
// evaluated as c1*me + c*(lo + up) with two TwoSums and exact scalings
// (17 flops instead of 31); the pair is kept unnormalized, which TwoSum
// tolerates, and is rounded to float once when stored.
template <bool Sym> struct CompensatedT {
  using V = DF;
  using Store = float;
  static __device__ __forceinline__ V load(Store x) { return {x, 0.0f}; }
  static __device__ __forceinline__ Store store(V x) {
    return __fadd_rn(x.h, x.l);
  }
  // Wavelet schedules may run the fine levels on packed pairs (sym_update2).
  static constexpr bool kPacked = Sym;

  template <bool C1>
  static __device__ __forceinline__ V update(Coeffs const &c, V lo, V me,
                                             V up) {
    if constexpr (Sym) {
      float const cc = c.f0;
      DF const s = two_sum(lo.h, up.h);
      float const e1 = __fadd_rn(s.l, __fadd_rn(lo.l, up.l));
      float const t = __fmul_rn(cc, s.h);
      float const m = C1 ? me.h : __fmul_rn(c.f1, me.h);
      DF const r = two_sum(m, t);
      float l = __fmaf_rn(cc, e1, r.l);
      l = C1 ? __fadd_rn(l, me.l) : __fmaf_rn(c.f1, me.l, l);
      return {r.h, l};
    } else {
      DF p0 = df_scale(c.f0, lo);
      DF p1 = C1 ? me : df_scale(c.f1, me);
      DF p2 = df_scale(c.f2, up);
      return df_add(df_add(p0, p1), p2);
    }
  }
};
using Compensated = CompensatedT<false>;
using CompensatedSym = CompensatedT<true>;

// ---------------------------------------------------------------------------
// Packed pairs of floats for the f32x2 instructions of sm_100+ (one issue
// slot computes two lanes' values). A pair lives in one 64-bit register.
using f2 = unsigned long long;

__device__ __forceinline__ f2 f2_pack(float x, float y) {
  f2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(x), "f"(y));
  return r;
}
__device__ __forceinline__ float f2_x(f2 r) {
  float x;
  asm("{\n\t.reg .f32 t;\n\tmov.b64 {%0, t}, %1;\n\t}" : "=f"(x) : "l"(r));
  return x;
}
__device__ __forceinline__ float f2_y(f2 r) {
  float y;
  asm("{\n\t.reg .f32 t;\n\tmov.b64 {t, %0}, %1;\n\t}" : "=f"(y) : "l"(r));
  return y;
}
__device__ __forceinline__ f2 f2_add(f2 a, f2 b) {
  f2 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2 f2_sub(f2 a, f2 b) {
  f2 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b) {
  f2 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2 f2_fma(f2 a, f2 b, f2 c) {
  f2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

// A pair of equal floats, built with integer operations so that the
// compiler folds it when x is a constant.
__device__ __forceinline__ f2 f2_splat(float x) {
  unsigned long long const b = __float_as_uint(x);
  return b | (b << 32);
}
// A pair from two raw 32-bit words (x in the low half) and back, as
// register-pair moves (no integer arithmetic).
__device__ __forceinline__ f2 f2_bits(unsigned x, unsigned y) {
  f2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "r"(x), "r"(y));
  return r;
}
__device__ __forceinline__ unsigned f2_lo(f2 r) {
  unsigned x;
  asm("{\n\t.reg .b32 t;\n\tmov.b64 {%0, t}, %1;\n\t}" : "=r"(x) : "l"(r));
  return x;
}
__device__ __forceinline__ unsigned f2_hi(f2 r) {
  unsigned y;
  asm("{\n\t.reg .b32 t;\n\tmov.b64 {t, %0}, %1;\n\t}" : "=r"(y) : "l"(r));
  return y;
}

// Two double-float values (h.x + l.x, h.y + l.y).
struct DF2 {
  f2 h, l;
};

__device__ __forceinline__ DF2 two_sum2(f2 a, f2 b) {
  f2 const s = f2_add(a, b);
  f2 const bb = f2_sub(s, a);
  f2 const e = f2_add(f2_sub(a, f2_sub(s, bb)), f2_sub(b, bb));
  return {s, e};
}

// The symmetric exact-scaler update of CompensatedT<true> on two values at
// once (same operations, same roundings per lane).
template <bool C1>
__device__ __forceinline__ DF2 sym_update2(Coeffs const &c, DF2 lo, DF2 me,
                                           DF2 up) {
  f2 const cc = f2_splat(c.f0);
  DF2 const s = two_sum2(lo.h, up.h);
  f2 const e1 = f2_add(s.l, f2_add(lo.l, up.l));
  f2 const t = f2_mul(cc, s.h);
  f2 m = me.h;
  if constexpr (!C1) m = f2_mul(f2_splat(c.f1), me.h);
  DF2 const r = two_sum2(m, t);
  f2 l = f2_fma(cc, e1, r.l);
  if constexpr (C1)
    l = f2_add(l, me.l);
  else
    l = f2_fma(f2_splat(c.f1), me.l, l);
  return {r.h, l};
}

// ---------------------------------------------------------------------------
// Rows of adjacent columns, for the wide kernel (lift.cuh). A thread holds
// kCols adjacent pencils of a strided axis; one value V is the row of kCols
// points at the same pencil position, loaded and stored as one vector
// (Store), and every operation acts on each column exactly as the scalar
// policy named below does, so results are bit-identical to it.

// Plain<float, true> on four columns: two f32x2 pairs (columns 0-1, 2-3).
struct F32Row4 {
  f2 a, b;
};
struct RowF32 {
  using V = F32Row4;
  using Store = uint4;
  using Elem = float;
  static constexpr int kCols = 4;
  static constexpr bool kPacked = false;
  static __device__ __forceinline__ V load(Store u) {
    return {f2_bits(u.x, u.y), f2_bits(u.z, u.w)};
  }
  static __device__ __forceinline__ Store store(V v) {
    return {f2_lo(v.a), f2_hi(v.a), f2_lo(v.b), f2_hi(v.b)};
  }
  // fma(c2, up, fma(c0, lo, c1 * me)) per column (Plain<float, true>).
  template <bool C1>
  static __device__ __forceinline__ f2 pair(Coeffs const &c, f2 lo, f2 me,
                                            f2 up) {
    f2 t = C1 ? me : f2_mul(f2_splat(c.f1), me);
    t = f2_fma(f2_splat(c.f0), lo, t);
    return f2_fma(f2_splat(c.f2), up, t);
  }
  template <bool C1>
  static __device__ __forceinline__ V update(Coeffs const &c, V lo, V me,
                                             V up) {
    return {pair<C1>(c, lo.a, me.a, up.a), pair<C1>(c, lo.b, me.b, up.b)};
  }
};

// CompensatedT<true> on two columns: one DF2 (sym_update2).
struct RowF32C {
  using V = DF2;
  using Store = uint2;
  using Elem = float;
  static constexpr int kCols = 2;
  static constexpr bool kPacked = false;
  static __device__ __forceinline__ V load(Store u) {
    return {f2_bits(u.x, u.y), 0ull};
  }
  static __device__ __forceinline__ Store store(V v) {
    f2 const s = f2_add(v.h, v.l);
    return {f2_lo(s), f2_hi(s)};
  }
  template <bool C1>
  static __device__ __forceinline__ V update(Coeffs const &c, V lo, V me,
                                             V up) {
    return sym_update2<C1>(c, lo, me, up);
  }
};

// Plain<double, true> on two columns.
struct F64Row2 {
  double x, y;
};
struct RowF64 {
  using V = F64Row2;
  using Store = double2;
  using Elem = double;
  static constexpr int kCols = 2;
  static constexpr bool kPacked = false;
  static __device__ __forceinline__ V load(Store u) { return {u.x, u.y}; }
  static __device__ __forceinline__ Store store(V v) { return {v.x, v.y}; }
  template <bool C1>
  static __device__ __forceinline__ V update(Coeffs const &c, V lo, V me,
                                             V up) {
    using P = Plain<double, true>;
    return {P::template update<C1>(c, lo.x, me.x, up.x),
            P::template update<C1>(c, lo.y, me.y, up.y)};
  }
};

} // namespace pgb
