/*****************************************************************************
 *
 *  lgb_vf2.cuh
 *
 *  vf2: the values of two lattice sites in one 64-bit register pair,
 *  computed with the packed FP32x2 instructions of sm_100 and later
 *  (__fadd2_rn, __fmul2_rn, __ffma2_rn: one instruction for both sites).
 *  The arithmetic operators make the per-site code of the reduced-precision
 *  step (templated on its number type) run two sites at a time.  A product
 *  is held as an unevaluated vmul so that a product followed by an
 *  addition becomes one packed fused multiply-add, as the scalar code
 *  contracts a*b + c; the error-free splittings of the mass sums use
 *  additions only, which are never contracted.
 *
 *****************************************************************************/

#ifndef LGB_VF2_CUH
#define LGB_VF2_CUH

#include <cuda_runtime.h>

struct vmul;

struct vf2 {
  float2 v;
  __device__ __forceinline__ vf2() {}
  __device__ __forceinline__ vf2(float2 a) : v(a) {}
  __device__ __forceinline__ vf2(float a, float b) : v(make_float2(a, b)) {}
  /* broadcast of a constant or a uniform parameter */
  __device__ __forceinline__ vf2(float a) : v(make_float2(a, a)) {}
  __device__ __forceinline__ explicit vf2(double a)
    : v(make_float2((float) a, (float) a)) {}
  __device__ __forceinline__ vf2(const vmul & m);
  __device__ __forceinline__ vf2 & operator=(const vmul & m);
  __device__ __forceinline__ vf2 & operator+=(const vf2 & b);
  __device__ __forceinline__ vf2 & operator-=(const vf2 & b);
  __device__ __forceinline__ vf2 & operator+=(const vmul & m);
  __device__ __forceinline__ vf2 & operator-=(const vmul & m);
  __device__ __forceinline__ vf2 & operator*=(const vf2 & b);
};

/* a*b, not yet rounded */
struct vmul {
  float2 a, b;
  __device__ __forceinline__ vmul(float2 x, float2 y) : a(x), b(y) {}
  __device__ __forceinline__ float2 eval() const { return __fmul2_rn(a, b); }
};

__device__ __forceinline__ vf2::vf2(const vmul & m) : v(m.eval()) {}
__device__ __forceinline__ vf2 & vf2::operator=(const vmul & m) {
  v = m.eval();
  return *this;
}

__device__ __forceinline__ float2 neg2(float2 a) {
  return make_float2(-a.x, -a.y);
}

__device__ __forceinline__ vmul operator*(const vf2 & a, const vf2 & b) {
  return vmul(a.v, b.v);
}
__device__ __forceinline__ vmul operator*(const vmul & m, const vf2 & b) {
  return vmul(m.eval(), b.v);
}
__device__ __forceinline__ vmul operator*(const vf2 & a, const vmul & m) {
  return vmul(a.v, m.eval());
}
__device__ __forceinline__ vmul operator*(const vmul & m, const vmul & n) {
  return vmul(m.eval(), n.eval());
}

__device__ __forceinline__ vf2 operator+(const vf2 & a, const vf2 & b) {
  return vf2(__fadd2_rn(a.v, b.v));
}
__device__ __forceinline__ vf2 operator-(const vf2 & a, const vf2 & b) {
  return vf2(__fadd2_rn(a.v, neg2(b.v)));
}
__device__ __forceinline__ vf2 operator-(const vf2 & a) {
  return vf2(neg2(a.v));
}
__device__ __forceinline__ vf2 operator-(const vmul & m) {
  return vf2(neg2(m.eval()));
}

/* products followed by a sum: one fused multiply-add */
__device__ __forceinline__ vf2 operator+(const vmul & m, const vf2 & c) {
  return vf2(__ffma2_rn(m.a, m.b, c.v));
}
__device__ __forceinline__ vf2 operator+(const vf2 & c, const vmul & m) {
  return vf2(__ffma2_rn(m.a, m.b, c.v));
}
__device__ __forceinline__ vf2 operator-(const vmul & m, const vf2 & c) {
  return vf2(__ffma2_rn(m.a, m.b, neg2(c.v)));
}
__device__ __forceinline__ vf2 operator-(const vf2 & c, const vmul & m) {
  return vf2(__ffma2_rn(neg2(m.a), m.b, c.v));
}
__device__ __forceinline__ vf2 operator+(const vmul & m, const vmul & n) {
  return vf2(__ffma2_rn(m.a, m.b, n.eval()));
}
__device__ __forceinline__ vf2 operator-(const vmul & m, const vmul & n) {
  return vf2(__ffma2_rn(m.a, m.b, neg2(n.eval())));
}

__device__ __forceinline__ vf2 & vf2::operator+=(const vf2 & b) {
  v = __fadd2_rn(v, b.v);
  return *this;
}
__device__ __forceinline__ vf2 & vf2::operator-=(const vf2 & b) {
  v = __fadd2_rn(v, neg2(b.v));
  return *this;
}
__device__ __forceinline__ vf2 & vf2::operator+=(const vmul & m) {
  v = __ffma2_rn(m.a, m.b, v);
  return *this;
}
__device__ __forceinline__ vf2 & vf2::operator-=(const vmul & m) {
  v = __ffma2_rn(neg2(m.a), m.b, v);
  return *this;
}
__device__ __forceinline__ vf2 & vf2::operator*=(const vf2 & b) {
  v = __fmul2_rn(v, b.v);
  return *this;
}

/* 1/a, lane by lane (IEEE division) */
__device__ __forceinline__ vf2 operator/(const vf2 & a, const vf2 & b) {
  return vf2(a.v.x/b.v.x, a.v.y/b.v.y);
}

/* c ? a : b, lane by lane, for c = (u > 0) and (u < 0) */
__device__ __forceinline__ vf2 sel_gt0(const vf2 & u, const vf2 & a,
				       const vf2 & b) {
  return vf2((u.v.x > 0.0f) ? a.v.x : b.v.x, (u.v.y > 0.0f) ? a.v.y : b.v.y);
}
__device__ __forceinline__ vf2 sel_lt0(const vf2 & u, const vf2 & a,
				       const vf2 & b) {
  return vf2((u.v.x < 0.0f) ? a.v.x : b.v.x, (u.v.y < 0.0f) ? a.v.y : b.v.y);
}

/*****************************************************************************
 *
 *  sf1: one site with exactly the roundings of a vf2 lane (each product
 *  rounded unless an addition follows, which then fuses with it; no other
 *  contraction), so that a value computed for one site alone equals the
 *  same value computed in a pair.
 *
 *****************************************************************************/

struct smul;

struct sf1 {
  float v;
  __device__ __forceinline__ sf1() {}
  __device__ __forceinline__ sf1(float a) : v(a) {}
  __device__ __forceinline__ explicit sf1(double a) : v((float) a) {}
  __device__ __forceinline__ sf1(const smul & m);
  __device__ __forceinline__ sf1 & operator=(const smul & m);
};

struct smul {
  float a, b;
  __device__ __forceinline__ smul(float x, float y) : a(x), b(y) {}
  __device__ __forceinline__ float eval() const { return __fmul_rn(a, b); }
};

__device__ __forceinline__ sf1::sf1(const smul & m) : v(m.eval()) {}
__device__ __forceinline__ sf1 & sf1::operator=(const smul & m) {
  v = m.eval();
  return *this;
}

__device__ __forceinline__ smul operator*(const sf1 & a, const sf1 & b) {
  return smul(a.v, b.v);
}
__device__ __forceinline__ smul operator*(const smul & m, const sf1 & b) {
  return smul(m.eval(), b.v);
}
__device__ __forceinline__ smul operator*(const sf1 & a, const smul & m) {
  return smul(a.v, m.eval());
}
__device__ __forceinline__ smul operator*(const smul & m, const smul & n) {
  return smul(m.eval(), n.eval());
}
__device__ __forceinline__ sf1 operator+(const sf1 & a, const sf1 & b) {
  return sf1(__fadd_rn(a.v, b.v));
}
__device__ __forceinline__ sf1 operator-(const sf1 & a, const sf1 & b) {
  return sf1(__fadd_rn(a.v, -b.v));
}
__device__ __forceinline__ sf1 operator-(const sf1 & a) { return sf1(-a.v); }
__device__ __forceinline__ sf1 operator+(const smul & m, const sf1 & c) {
  return sf1(__fmaf_rn(m.a, m.b, c.v));
}
__device__ __forceinline__ sf1 operator+(const sf1 & c, const smul & m) {
  return sf1(__fmaf_rn(m.a, m.b, c.v));
}
__device__ __forceinline__ sf1 operator-(const smul & m, const sf1 & c) {
  return sf1(__fmaf_rn(m.a, m.b, -c.v));
}
__device__ __forceinline__ sf1 operator-(const sf1 & c, const smul & m) {
  return sf1(__fmaf_rn(-m.a, m.b, c.v));
}
__device__ __forceinline__ sf1 operator+(const smul & m, const smul & n) {
  return sf1(__fmaf_rn(m.a, m.b, n.eval()));
}
__device__ __forceinline__ sf1 operator-(const smul & m, const smul & n) {
  return sf1(__fmaf_rn(m.a, m.b, -n.eval()));
}

#endif
