// Paired FP32 arithmetic for sm_100-family GPUs: a value type F2 holding two
// lanes of a computation, whose +, -, * map onto the paired instructions
// (__fadd2_rn, __fmul2_rn, __ffma2_rn: one issue slot for two operations).
//
// A product is kept pending (F2P) until it is added to or subtracted from
// something, so `a * b + c` becomes one fused paired multiply-add, the way the
// compiler contracts the scalar expression.  The stencil templates of
// sph_core.cuh instantiate unchanged with T = F2, so a thread evaluates the
// same expressions for two points at once.
#pragma once
#include <cuda_runtime.h>

namespace sph {

struct F2 {
    float2 v;
    __device__ __forceinline__ F2() {}
    __device__ __forceinline__ F2(float2 x) : v(x) {}
    __device__ __forceinline__ F2(float a, float b) : v(make_float2(a, b)) {}
    __device__ __forceinline__ F2(float x) : v(make_float2(x, x)) {}
    __device__ __forceinline__ F2(double x) : v(make_float2((float)x, (float)x)) {}
    __device__ __forceinline__ F2(int x) : v(make_float2((float)x, (float)x)) {}
};

__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

struct F2P {  // pending product a * b
    float2 a, b;
    __device__ __forceinline__ operator F2() const { return F2(__fmul2_rn(a, b)); }
};

__device__ __forceinline__ F2 operator+(F2 x, F2 y) { return F2(__fadd2_rn(x.v, y.v)); }
__device__ __forceinline__ F2 operator-(F2 x, F2 y) { return F2(__fadd2_rn(x.v, neg2(y.v))); }
__device__ __forceinline__ F2 operator-(F2 x) { return F2(neg2(x.v)); }
__device__ __forceinline__ F2P operator*(F2 x, F2 y) { return F2P{x.v, y.v}; }
__device__ __forceinline__ F2P operator*(F2P p, F2 c) { return F2P{__fmul2_rn(p.a, p.b), c.v}; }
__device__ __forceinline__ F2P operator*(F2 c, F2P p) { return F2P{c.v, __fmul2_rn(p.a, p.b)}; }
__device__ __forceinline__ F2P operator*(F2P p, F2P q) { return F2P{__fmul2_rn(p.a, p.b), __fmul2_rn(q.a, q.b)}; }
__device__ __forceinline__ F2 operator+(F2P p, F2 c) { return F2(__ffma2_rn(p.a, p.b, c.v)); }
__device__ __forceinline__ F2 operator+(F2 c, F2P p) { return F2(__ffma2_rn(p.a, p.b, c.v)); }
__device__ __forceinline__ F2 operator+(F2P p, F2P q) { return F2(__ffma2_rn(p.a, p.b, __fmul2_rn(q.a, q.b))); }
__device__ __forceinline__ F2 operator-(F2P p, F2 c) { return F2(__ffma2_rn(p.a, p.b, neg2(c.v))); }
__device__ __forceinline__ F2 operator-(F2 c, F2P p) { return F2(__ffma2_rn(neg2(p.a), p.b, c.v)); }
__device__ __forceinline__ F2 operator-(F2P p, F2P q) { return F2(__ffma2_rn(p.a, p.b, neg2(__fmul2_rn(q.a, q.b)))); }

// fast quotient per lane (the FP32 pdiv of sph_core.cuh)
__device__ __forceinline__ F2 pdiv(F2 a, F2 b) { return F2(__fdividef(a.v.x, b.v.x), __fdividef(a.v.y, b.v.y)); }

// keep lane 0 / lane 1 or zero it
__device__ __forceinline__ F2 keep(F2 x, bool m0, bool m1) { return F2(m0 ? x.v.x : 0.f, m1 ? x.v.y : 0.f); }

}  // namespace sph
