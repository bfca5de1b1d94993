// move_f32.cuh -- FP32 trial moves of the device-resident chains.
//
// A chain molecule is held as: anchor (its first primary atom) in 32-bit
// fixed point of the box edge, a unit quaternion q (FP32), and per atom a
// template offset t_a (the offset from the anchor at the start, FP32) and
// its current offset o_a = R(q) t_a.  A trial move about the vertex atom v
// with rotation R_d and translation d gives
//     q' = normalise(q_d * q),  o'_a = R(q') t_a,
//     anchor' = anchor + fix(o_v - o'_v + d),
// which is the reference's move (rotate every atom about the vertex,
// translate, SimulationStep.cpp:544-565) in exact arithmetic.  The anchor
// wraps modulo the box edge like keepMoleculeInBox (:710-729).  There is no
// FP64 in a move (GB300 issues FP64 at 1/64 of FP32), the rigid geometry
// does not drift (offsets are always R(q) applied to the template), and
// every operation is an explicitly rounded FP32 operation, so a CPU mirror
// reproduces the state bit for bit.
#pragma once

#include "device.cuh"

namespace mcgpu {

// Uniform in (0, 1) as a float from 32 random bits: 24 bits, exact.
__device__ __forceinline__ float u01f(unsigned r) {
  return __fmaf_rn((float)(r >> 8), 5.9604644775390625e-08f, 2.98023223876953125e-08f);
}

// sin and cos of x (|x| <= 8 pi): x = k pi/2 + r with a three-part pi/2
// (Cody and Waite's reduction), |r| <= pi/4, then the Taylor polynomials of
// sin r (to r^11) and cos r (to r^12), evaluated by Horner's rule with
// explicit fused multiply-adds; quadrant k mod 4 picks the signs.
__device__ __forceinline__ void sincos_f32(float x, float* sp, float* cp) {
  const float k = rintf(__fmul_rn(x, 0.636619772367581343f));
  float r = __fmaf_rn(-k, 1.5703125f, x);
  r = __fmaf_rn(-k, 4.83751296997070312e-04f, r);
  r = __fmaf_rn(-k, 7.54978995489188216e-08f, r);
  const float r2 = __fmul_rn(r, r);
  float s = __fmaf_rn(r2, -2.50521083854417188e-08f, 2.75573192239858907e-06f);
  s = __fmaf_rn(r2, s, -1.98412698412698413e-04f);
  s = __fmaf_rn(r2, s, 8.33333333333333333e-03f);
  s = __fmaf_rn(r2, s, -1.66666666666666667e-01f);
  s = __fmaf_rn(__fmul_rn(r2, r), s, r);
  float c = __fmaf_rn(r2, 2.08767569878680990e-09f, -2.75573192239858907e-07f);
  c = __fmaf_rn(r2, c, 2.48015873015873016e-05f);
  c = __fmaf_rn(r2, c, -1.38888888888888889e-03f);
  c = __fmaf_rn(r2, c, 4.16666666666666667e-02f);
  c = __fmaf_rn(r2, c, -0.5f);
  c = __fmaf_rn(r2, c, 1.0f);
  const int q = ((int)k) & 3;
  const float ss = (q == 0) ? s : (q == 1) ? c : (q == 2) ? -s : -c;
  const float cc = (q == 0) ? c : (q == 1) ? -s : (q == 2) ? -c : s;
  *sp = ss;
  *cp = cc;
}

struct QuatF {
  float w, x, y, z;
};

// Hamilton product a * b (rotation b first, then a).
__device__ __forceinline__ QuatF qmul(QuatF a, QuatF b) {
  QuatF r;
  r.w = __fsub_rn(__fsub_rn(__fsub_rn(__fmul_rn(a.w, b.w), __fmul_rn(a.x, b.x)), __fmul_rn(a.y, b.y)),
                  __fmul_rn(a.z, b.z));
  r.x = __fsub_rn(__fadd_rn(__fadd_rn(__fmul_rn(a.w, b.x), __fmul_rn(a.x, b.w)), __fmul_rn(a.y, b.z)),
                  __fmul_rn(a.z, b.y));
  r.y = __fadd_rn(__fadd_rn(__fsub_rn(__fmul_rn(a.w, b.y), __fmul_rn(a.x, b.z)), __fmul_rn(a.y, b.w)),
                  __fmul_rn(a.z, b.x));
  r.z = __fadd_rn(__fsub_rn(__fadd_rn(__fmul_rn(a.w, b.z), __fmul_rn(a.x, b.y)), __fmul_rn(a.y, b.x)),
                  __fmul_rn(a.z, b.w));
  return r;
}

__device__ __forceinline__ QuatF qnormalise(QuatF a) {
  const float n2 = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(a.w, a.w), __fmul_rn(a.x, a.x)),
                                       __fmul_rn(a.y, a.y)),
                             __fmul_rn(a.z, a.z));
  const float n = __fsqrt_rn(n2);
  QuatF r;
  r.w = __fdiv_rn(a.w, n);
  r.x = __fdiv_rn(a.x, n);
  r.y = __fdiv_rn(a.y, n);
  r.z = __fdiv_rn(a.z, n);
  return r;
}

// Rotation matrix of a unit quaternion, row-major.
__device__ __forceinline__ void qmatrix(QuatF q, float* m) {
  const float xx = __fmul_rn(q.x, q.x), yy = __fmul_rn(q.y, q.y), zz = __fmul_rn(q.z, q.z);
  const float xy = __fmul_rn(q.x, q.y), xz = __fmul_rn(q.x, q.z), yz = __fmul_rn(q.y, q.z);
  const float wx = __fmul_rn(q.w, q.x), wy = __fmul_rn(q.w, q.y), wz = __fmul_rn(q.w, q.z);
  m[0] = __fsub_rn(1.0f, __fmul_rn(2.0f, __fadd_rn(yy, zz)));
  m[1] = __fmul_rn(2.0f, __fsub_rn(xy, wz));
  m[2] = __fmul_rn(2.0f, __fadd_rn(xz, wy));
  m[3] = __fmul_rn(2.0f, __fadd_rn(xy, wz));
  m[4] = __fsub_rn(1.0f, __fmul_rn(2.0f, __fadd_rn(xx, zz)));
  m[5] = __fmul_rn(2.0f, __fsub_rn(yz, wx));
  m[6] = __fmul_rn(2.0f, __fsub_rn(xz, wy));
  m[7] = __fmul_rn(2.0f, __fadd_rn(yz, wx));
  m[8] = __fsub_rn(1.0f, __fmul_rn(2.0f, __fadd_rn(xx, yy)));
}

__device__ __forceinline__ float3 mvec(const float* m, float x, float y, float z) {
  return make_float3(__fadd_rn(__fadd_rn(__fmul_rn(m[0], x), __fmul_rn(m[1], y)), __fmul_rn(m[2], z)),
                     __fadd_rn(__fadd_rn(__fmul_rn(m[3], x), __fmul_rn(m[4], y)), __fmul_rn(m[5], z)),
                     __fadd_rn(__fadd_rn(__fmul_rn(m[6], x), __fmul_rn(m[7], y)), __fmul_rn(m[8], z)));
}

// Rotation quaternion about unit axis (kx, ky, kz) by angle a (radians).
__device__ __forceinline__ QuatF qaxis(float kx, float ky, float kz, float a) {
  float s, c;
  sincos_f32(__fmul_rn(0.5f, a), &s, &c);
  QuatF q;
  q.w = c;
  q.x = __fmul_rn(s, kx);
  q.y = __fmul_rn(s, ky);
  q.z = __fmul_rn(s, kz);
  return q;
}

// A device-drawn trial move in FP32.
struct MoveF {
  int mol, vertex;
  float dx, dy, dz;
  QuatF qd;       // rotation of the move (not normalised)
  float u;        // acceptance uniform in (0, 1)
};
static_assert(sizeof(MoveF) == kPropBytes, "MoveF size");

constexpr float kDeg2Rad = 0.0174532925199432958f;

// The move of (seed, chain, step).  Counter layout (step_lo, step_hi, chain,
// block): block 0 gives molecule, vertex, dx, dy; block 1 gives dz and the
// three rotation draws; block 2 gives the acceptance uniform.  Euler form:
// rotations about x, then y, then z by angles U(-maxR, maxR) degrees with
// the reference's sense (SimulationStep.cpp:400-422 turn by -angle in the
// right-handed convention).  Axis form: axis uniform on the sphere
// (z = 2u - 1, phi = 2 pi u'), angle U(-maxR, maxR) degrees.
__device__ inline MoveF draw_move_f32(unsigned long long seed, unsigned chain,
                                      unsigned long long step, int n_mol, const int* mlen_chain,
                                      float max_t, float max_r, int mode) {
  const uint2 key = make_uint2((unsigned)seed, (unsigned)(seed >> 32));
  const unsigned s0 = (unsigned)step, s1 = (unsigned)(step >> 32);
  const uint4 a = philox4x32_10(make_uint4(s0, s1, chain, 0u), key);
  const uint4 c = philox4x32_10(make_uint4(s0, s1, chain, 1u), key);
  const uint4 d = philox4x32_10(make_uint4(s0, s1, chain, 2u), key);
  MoveF mv;
  mv.mol = uidx(a.x, n_mol);
  mv.vertex = uidx(a.y, mlen_chain[mv.mol] & 255);
  const float t2 = __fmul_rn(2.0f, max_t);
  mv.dx = __fsub_rn(__fmul_rn(t2, u01f(a.z)), max_t);
  mv.dy = __fsub_rn(__fmul_rn(t2, u01f(a.w)), max_t);
  mv.dz = __fsub_rn(__fmul_rn(t2, u01f(c.x)), max_t);
  const float r2 = __fmul_rn(2.0f, max_r);
  if (mode == MCGPU_ROT_EULER) {
    const float ax = __fmul_rn(__fsub_rn(__fmul_rn(r2, u01f(c.y)), max_r), kDeg2Rad);
    const float ay = __fmul_rn(__fsub_rn(__fmul_rn(r2, u01f(c.z)), max_r), kDeg2Rad);
    const float az = __fmul_rn(__fsub_rn(__fmul_rn(r2, u01f(c.w)), max_r), kDeg2Rad);
    const QuatF qx = qaxis(-1.0f, 0.0f, 0.0f, ax);
    const QuatF qy = qaxis(0.0f, -1.0f, 0.0f, ay);
    const QuatF qz = qaxis(0.0f, 0.0f, -1.0f, az);
    mv.qd = qmul(qz, qmul(qy, qx));
  } else {
    const float zc = __fsub_rn(__fmul_rn(2.0f, u01f(c.y)), 1.0f);
    const float phi = __fmul_rn(6.28318530717958648f, u01f(c.z));
    const float sr = __fsqrt_rn(__fsub_rn(1.0f, __fmul_rn(zc, zc)));
    float sp, cp;
    sincos_f32(phi, &sp, &cp);
    const float ang = __fmul_rn(__fsub_rn(__fmul_rn(r2, u01f(c.w)), max_r), kDeg2Rad);
    mv.qd = qaxis(__fmul_rn(sr, cp), __fmul_rn(sr, sp), zc, ang);
  }
  mv.u = u01f(d.x);
  return mv;
}

// Fixed-point step of a small FP32 displacement (|dx| < L/2).
__device__ __forceinline__ int fixstep(float dx, float inv_s) {
  return __float2int_rn(__fmul_rn(dx, inv_s));
}

}  // namespace mcgpu
