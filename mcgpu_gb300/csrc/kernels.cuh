// kernels.cuh -- the group-level pieces shared by every kernel: staging of
// the moved molecule, the cutoff screen, the per-warp neighbour rings, the
// pair batches (FP32 pair terms with FP64 per-neighbour sums, or FP64 pair
// terms), reductions and the commit.
#pragma once

#include "device.cuh"

namespace mcgpu {

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Primary position wrapped into [0, L) (FP32), for the screen.
__device__ __forceinline__ float4 wrap_pos(double x, double y, double z, const ChainHdr& H) {
  double wx = x - H.L[0] * floor(x / H.L[0]);
  double wy = y - H.L[1] * floor(y / H.L[1]);
  double wz = z - H.L[2] * floor(z / H.L[2]);
  return make_float4((float)wx, (float)wy, (float)wz, 0.f);
}

// Anchor position in 32-bit fixed point of the box edge (wraps mod 2^32).
__device__ __forceinline__ uint4 fixpos(double x, double y, double z, const ChainHdr& H) {
  return make_uint4((unsigned)(unsigned long long)__double2ll_rn(x * H.fxinv[0]),
                    (unsigned)(unsigned long long)__double2ll_rn(y * H.fxinv[1]),
                    (unsigned)(unsigned long long)__double2ll_rn(z * H.fxinv[2]), 0u);
}

// Minimum-image anchor difference b - a in Angstrom (FP32).
__device__ __forceinline__ float3 fixdiff(uint4 b, uint4 a, const ChainHdr& H) {
  return make_float3((float)(int)(b.x - a.x) * H.fxs[0], (float)(int)(b.y - a.y) * H.fxs[1],
                     (float)(int)(b.z - a.z) * H.fxs[2]);
}

// The same difference as a double-float (hi + lo), exact to ~1e-14 A: the
// fixed-point difference is split into a high part with its low 8 bits
// cleared (exact in FP32) and the rest, each scaled by L/2^32 held as
// fxs + fxs_lo, with the rounding of the main product recovered by an FMA.
__device__ __forceinline__ void fixdiff_ff(uint4 b, uint4 a, const ChainHdr& H, float3& hi,
                                           float3& lo) {
  const int d[3] = {(int)(b.x - a.x), (int)(b.y - a.y), (int)(b.z - a.z)};
  float h[3], l[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const int dh = d[k] & ~0xFF;
    const float fh = (float)dh, fl = (float)(d[k] - dh);
    const float p = fh * H.fxs[k];
    const float e = fmaf(fh, H.fxs[k], -p);
    const float t = fmaf(fh, H.fxs_lo[k], fmaf(fl, H.fxs[k], e));
    h[k] = p + t;
    l[k] = t - (h[k] - p);
  }
  hi = make_float3(h[0], h[1], h[2]);
  lo = make_float3(l[0], l[1], l[2]);
}

// True when an atom pair of these two molecules may need its own periodic
// image (|D| + radii reaches half a box edge in some dimension).
__device__ __forceinline__ bool needs_wrap(float3 D, float rr, const ChainHdr& H) {
  return fabsf(D.x) + rr > 0.5f * H.Lf[0] - 1e-3f || fabsf(D.y) + rr > 0.5f * H.Lf[1] - 1e-3f ||
         fabsf(D.z) + rr > 0.5f * H.Lf[2] - 1e-3f;
}

// The reference's cutoff test for one primary pair, FP64, same rounding
// (SimulationStep.cpp:325-326 with :332-342 and :377-385).
__device__ __forceinline__ bool in_range64(double x1, double y1, double z1, int p2,
                                           const Pool& P, const ChainHdr& H) {
  double dx = make_periodic(P.x[p2] - x1, H.L[0]);
  double dy = make_periodic(P.y[p2] - y1, H.L[1]);
  double dz = make_periodic(P.z[p2] - z1, H.L[2]);
  double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
  return r2 <= __dmul_rn(H.cutoff, H.cutoff);
}

__device__ __forceinline__ float r2_screen(float4 a, float4 b, const ChainHdr& H) {
  float dx = wrapf(b.x - a.x, H.Lf[0]);
  float dy = wrapf(b.y - a.y, H.Lf[1]);
  float dz = wrapf(b.z - a.z, H.Lf[2]);
  return fmaf(dx, dx, fmaf(dy, dy, dz * dz));
}

// ---- staging ------------------------------------------------------------

// misc[] slots of the staged molecule's FP32 radius and net charge factor
// (float bits: no FP64 on the step's path).
enum : int { kMiscRad = 21, kMiscQm = 22 };

// Lanes of ONE warp stage molecule m: its current placement ("old") and, if
// p is non-null, the proposed placement ("new") computed as
// SimCalcs::intermolecularMove does (SimulationStep.cpp:544-565): every
// non-vertex atom rotated about the vertex and translated, the vertex
// translated, then the molecule wrapped by its first primary atom
// (keepMoleculeInBox, :710-729).  Results go to shared memory; scalars to
// misc/miscd.  The caller synchronises the group afterwards.
__device__ inline void stage(const Pool& P, const ChainHdr& H, int m, const Proposal* p,
                      const GroupSmem& s, int lane) {
  const int a0 = P.mstart[m];
  const int lw = P.mlen[m];
  const int len = lw & 255;
  const int2 pi = P.mpi[m];
  for (int i = lane; i < len; i += 32) {
    int a = a0 + i;
    s.ox[i] = P.x[a]; s.oy[i] = P.y[a]; s.oz[i] = P.z[a];
    const double2 bl = blend64(P.sig[a], P.eps[a]);
    s.sd[i] = bl.x; s.ed[i] = bl.y; s.qd[i] = P.q[a];
    const float4 o = P.aoff[a];
    const float2 q = P.aeq[a];
    s.o_old[i] = o;
    s.l_old[i] = P.aofl[a];
    s.eq[i] = make_float4(q.x, q.y, fmaf(o.x, o.x, fmaf(o.y, o.y, o.z * o.z)), 0.f);
  }
  // net FP32 charge factor of the molecule (sum over lanes, fixed order)
  float qsum = 0.f;
  for (int i = lane; i < len; i += 32) qsum += P.aeq[a0 + i].y;
  for (int off = 16; off > 0; off >>= 1) qsum += __shfl_xor_sync(~0u, qsum, off);
  for (int k = lane; k < pi.y; k += 32) {
    s.p_old[k] = P.ppos[pi.x + k];
    s.pa[k] = P.pidx[pi.x + k] - a0;
  }
  uint4 fo = P.mfix[m];
  if (lane == 0) {
    s.misc[0] = m; s.misc[1] = a0; s.misc[2] = len; s.misc[3] = pi.y;
    s.misc[4] = lw >> 8; s.misc[5] = p ? 3 : 1; s.misc[6] = p ? p->vertex : -1;
    s.misc[8] = (int)fo.x; s.misc[9] = (int)fo.y; s.misc[10] = (int)fo.z;
    s.misc[kMiscRad] = __float_as_int(P.mrad[m]);
    s.misc[kMiscQm] = __float_as_int(qsum);
  }
  if (!p) return;
  Rot R;
  if (lane == 0) R = make_rot(*p);
  R.mode = p->mode;
  R.cx = __shfl_sync(~0u, R.cx, 0); R.sx = __shfl_sync(~0u, R.sx, 0);
  R.cy = __shfl_sync(~0u, R.cy, 0); R.sy = __shfl_sync(~0u, R.sy, 0);
  R.cz = __shfl_sync(~0u, R.cz, 0); R.sz = __shfl_sync(~0u, R.sz, 0);
  R.kx = __shfl_sync(~0u, R.kx, 0); R.ky = __shfl_sync(~0u, R.ky, 0);
  R.kz = __shfl_sync(~0u, R.kz, 0);
  __syncwarp();
  const int v = p->vertex;
  const double px = s.ox[v], py = s.oy[v], pz = s.oz[v];
  for (int i = lane; i < len; i += 32) {
    double x, y, z;
    if (i == v) {
      x = __dadd_rn(px, p->dx); y = __dadd_rn(py, p->dy); z = __dadd_rn(pz, p->dz);
    } else {
      double vx = __dadd_rn(s.ox[i], -px), vy = __dadd_rn(s.oy[i], -py), vz = __dadd_rn(s.oz[i], -pz);
      rot_apply(R, vx, vy, vz);
      x = __dadd_rn(__dadd_rn(vx, px), p->dx);
      y = __dadd_rn(__dadd_rn(vy, py), p->dy);
      z = __dadd_rn(__dadd_rn(vz, pz), p->dz);
    }
    s.nx[i] = x; s.ny[i] = y; s.nz[i] = z;
  }
  __syncwarp();
  const int an = s.pa[0];
  double ax = s.nx[an], ay = s.ny[an], az = s.nz[an];
  double shx = 0, shy = 0, shz = 0;
  if (ax < 0) shx = H.L[0]; else if (ax > H.L[0]) shx = -H.L[0];
  if (ay < 0) shy = H.L[1]; else if (ay > H.L[1]) shy = -H.L[1];
  if (az < 0) shz = H.L[2]; else if (az > H.L[2]) shz = -H.L[2];
  if (shx != 0) ax = __dadd_rn(ax, shx);
  if (shy != 0) ay = __dadd_rn(ay, shy);
  if (shz != 0) az = __dadd_rn(az, shz);
  __syncwarp();
  for (int i = lane; i < len; i += 32) {
    double x = s.nx[i], y = s.ny[i], z = s.nz[i];
    if (shx != 0) x = __dadd_rn(x, shx);
    if (shy != 0) y = __dadd_rn(y, shy);
    if (shz != 0) z = __dadd_rn(z, shz);
    s.nx[i] = x; s.ny[i] = y; s.nz[i] = z;
    const double vx = x - ax, vy = y - ay, vz = z - az;
    const float4 o = make_float4((float)vx, (float)vy, (float)vz, s.o_old[i].w);
    s.o_new[i] = o;
    s.l_new[i] = make_float4((float)(vx - (double)o.x), (float)(vy - (double)o.y),
                             (float)(vz - (double)o.z), 0.f);
    s.eq[i].w = fmaf(o.x, o.x, fmaf(o.y, o.y, o.z * o.z));
  }
  __syncwarp();
  for (int k = lane; k < pi.y; k += 32) {
    int q = s.pa[k];
    s.p_new[k] = wrap_pos(s.nx[q], s.ny[q], s.nz[q], H);
  }
  if (lane == 0) {
    uint4 fn = fixpos(ax, ay, az, H);
    s.misc[12] = (int)fn.x; s.misc[13] = (int)fn.y; s.misc[14] = (int)fn.z;
  }
}

__device__ __forceinline__ MovedInfo load_moved(const GroupSmem& s) {
  MovedInfo mi;
  mi.mol = s.misc[0]; mi.atom0 = s.misc[1]; mi.len = s.misc[2]; mi.npidx = s.misc[3];
  mi.act = s.misc[4]; mi.states = s.misc[5]; mi.vertex = s.misc[6]; mi.pad = 0;
  mi.fx_old = make_uint4((unsigned)s.misc[8], (unsigned)s.misc[9], (unsigned)s.misc[10], 0u);
  mi.fx_new = make_uint4((unsigned)s.misc[12], (unsigned)s.misc[13], (unsigned)s.misc[14], 0u);
  mi.rad = __int_as_float(s.misc[kMiscRad]);
  mi.qm = __int_as_float(s.misc[kMiscQm]);
  return mi;
}

// ---- screen ---------------------------------------------------------------

// FP32 screen with FP64 re-test inside the guard band (plain path: FP64
// positions from the master rows).
__device__ __forceinline__ int screen_mixed(const Pool& P, const ChainHdr& H, const GroupSmem& s,
                                            const MovedInfo& mi, int j) {
  const int2 pj = P.mpi[j];
  int f = 0;
  for (int k2 = 0; k2 < pj.y; k2++) {
    const float4 q = P.ppos[pj.x + k2];
    for (int k1 = 0; k1 < mi.npidx; k1++) {
      if ((mi.states & 1) && !(f & kInOld)) {
        float r2 = r2_screen(s.p_old[k1], q, H);
        if (r2 <= H.cut2_lo) {
          f |= kInOld;
        } else if (r2 <= H.cut2_hi) {
          int pa = s.pa[k1];
          if (in_range64(s.ox[pa], s.oy[pa], s.oz[pa], P.pidx[pj.x + k2], P, H)) f |= kInOld;
        }
      }
      if ((mi.states & 2) && !(f & kInNew)) {
        float r2 = r2_screen(s.p_new[k1], q, H);
        if (r2 <= H.cut2_lo) {
          f |= kInNew;
        } else if (r2 <= H.cut2_hi) {
          int pa = s.pa[k1];
          if (in_range64(s.nx[pa], s.ny[pa], s.nz[pa], P.pidx[pj.x + k2], P, H)) f |= kInNew;
        }
      }
    }
  }
  return f;
}

// FP64 screen: the reference's test for every primary pair.
__device__ __forceinline__ int screen_f64(const Pool& P, const ChainHdr& H, const GroupSmem& s,
                                          const MovedInfo& mi, int j) {
  const int2 pj = P.mpi[j];
  int f = 0;
  for (int k2 = 0; k2 < pj.y; k2++) {
    const int p2 = P.pidx[pj.x + k2];
    for (int k1 = 0; k1 < mi.npidx; k1++) {
      const int pa = s.pa[k1];
      if ((mi.states & 1) && !(f & kInOld) && in_range64(s.ox[pa], s.oy[pa], s.oz[pa], p2, P, H))
        f |= kInOld;
      if ((mi.states & 2) && !(f & kInNew) && in_range64(s.nx[pa], s.ny[pa], s.nz[pa], p2, P, H))
        f |= kInNew;
    }
  }
  return f;
}

// ---- pair batches -----------------------------------------------------------

// Per-thread double-float accumulators of one evaluation.
struct AccFF {
  float oh, ol, nh, nl, ab;
  long long np;
};

// Displacement of a pair, atom b of the neighbour minus atom a of the moved
// molecule, both anchor-relative to the moved molecule's anchor.  PRECISE
// adds the low parts (bl: of b = D + o_b; la: of a's offset) so the only
// rounding left is the final one at the displacement's own magnitude.
template <bool PRECISE>
__device__ __forceinline__ float3 pair_disp(float3 bh, float3 bl, float4 a, float4 la) {
  if (PRECISE)
    return make_float3((bh.x - a.x) + (bl.x - la.x), (bh.y - a.y) + (bl.y - la.y),
                       (bh.z - a.z) + (bl.z - la.z));
  return make_float3(bh.x - a.x, bh.y - a.y, bh.z - a.z);
}

// Sum over the moved molecule's atoms a of the FP32 pair terms with one
// neighbour atom b, per-pair periodic image (entries whose atom pairs may
// straddle half a box edge).  abs accumulates |LJ| + |Coulomb|.
//
// NLEN > 0 fixes the moved molecule's length (at most 4) at compile time:
// the loop unrolls so its independent pair terms interleave, and bit i of
// ljmask clear means the LJ term of moved atom i is exactly zero (a sigma or
// epsilon product of zero) and is not evaluated.  NLEN == 0 (any length up
// to 64) ignores ljmask.  Neither changes a bit of the sum.
template <bool PRECISE, int NLEN = 0>
__device__ __forceinline__ float sum_moved32_wrap(const float4* o, const float4* lo,
                                                  const float4* eq, int len, float3 bh, float3 bl,
                                                  float sb, float2 qb, const ChainHdr& H,
                                                  float& abs, unsigned ljmask = ~0u) {
  float acc = 0.f;
  auto term = [&](int i) {
    const float4 ea = eq[i];
    const float4 a = o[i];
    const float3 d = pair_disp<PRECISE>(bh, bl, a, PRECISE ? lo[i] : a);
    const float dx = wrapf(d.x, H.Lf[0]);
    const float dy = wrapf(d.y, H.Lf[1]);
    const float dz = wrapf(d.z, H.Lf[2]);
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    const float ir = rsqrt_nr(r2);
    const float lj = (NLEN == 0 || ((ljmask >> i) & 1u)) ? lj32(rcp_nr(r2), a.w, sb, ea.x, qb.x)
                                                         : 0.f;
    const float cl = (ea.y * qb.y) * ir;
    const bool ok = r2 > 0.f;
    acc += ok ? lj + cl : 0.f;
    abs += ok ? fabsf(lj) + fabsf(cl) : 0.f;
  };
  if (NLEN > 0) {
#pragma unroll
    for (int i = 0; i < (NLEN > 0 ? NLEN : 1); i++) term(i);
  } else {
    for (int i = 0; i < len; i++) term(i);
  }
  return acc;
}

// The same sum for an entry whose pairs all use the anchors' image, with
// the Coulomb part written for neutral molecules: with R = |b - anchor_m|,
//   sum_a q_a / r_ab = sum_a q_a (1/r_ab - 1/R) + Q_m / R,
//   1/r - 1/R = (R^2 - r^2) / (r R (r + R)),  R^2 - r^2 = 2 b.o_a - |o_a|^2,
// so every Coulomb term is O(|o_a| / R) smaller than q_a q_b / r and carries
// proportionally less FP32 rounding.  A coincident pair (r = 0) is skipped
// as the reference skips it (BruteForceStep.cpp:68-69).  use_new selects the
// |o_a|^2 of the placement (eq.z old, eq.w new).
template <bool PRECISE, int NLEN = 0>
__device__ __forceinline__ float sum_moved32_cf(const float4* o, const float4* lo,
                                                const float4* eq, int len, bool use_new,
                                                float3 bh, float3 bl, float sb, float2 qb,
                                                float qm, float& abs, unsigned ljmask = ~0u) {
  const float R2 = fmaf(bh.x, bh.x, fmaf(bh.y, bh.y, bh.z * bh.z));
  const float iR = rsqrt_nr(R2);
  const float R = R2 * iR;
  const float tx = bh.x + bh.x, ty = bh.y + bh.y, tz = bh.z + bh.z;
  float lj_acc = 0.f, phi = 0.f, lj_abs = 0.f, c_abs = 0.f;
  auto term = [&](int i) {
    const float4 a = o[i];
    const float4 ea = eq[i];
    const float3 d = pair_disp<PRECISE>(bh, bl, a, PRECISE ? lo[i] : a);
    const float r2 = fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z));
    const float ir = rsqrt_nr(r2);
    const float lj = (NLEN == 0 || ((ljmask >> i) & 1u)) ? lj32(rcp_nr(r2), a.w, sb, ea.x, qb.x)
                                                         : 0.f;
    const float num = fmaf(tx, a.x, fmaf(ty, a.y, fmaf(tz, a.z, -(use_new ? ea.w : ea.z))));
    const float w = ir * rcp_approx(fmaf(r2, ir, R));
    const bool ok = r2 > 0.f;
    const float c = ok ? (ea.y * num) * w : -ea.y;
    lj_acc += ok ? lj : 0.f;
    lj_abs += ok ? fabsf(lj) : 0.f;
    phi += c;
    c_abs += fabsf(c);
  };
  if (NLEN > 0) {
#pragma unroll
    for (int i = 0; i < (NLEN > 0 ? NLEN : 1); i++) term(i);
  } else {
    for (int i = 0; i < len; i++) term(i);
  }
  const float f = qb.y * iR;
  abs += lj_abs + fabsf(f) * (c_abs + fabsf(qm));
  return fmaf(f, phi + qm, lj_acc);
}

// Pair batch of `count` ring entries from `head`, teams of T lanes (T a
// power of two <= 32): the team forms the entry's anchor differences
// (fixed point -> FP32, or double-float when PRECISE) and image flags, lane
// tl takes neighbour atoms tl, tl+T, ... against every atom of the moved
// molecule, and the team's FP32 partial of the entry is added in
// double-float to the team leader's accumulators.  LO: the plain path, whose
// FP32 offsets carry low parts (aofl, l_old/l_new).
template <bool PRECISE, bool LO>
__device__ __forceinline__ void batch_ff(const Pool& P, const ChainHdr& H, const GroupSmem& s,
                                         const MovedInfo& mi, const int* rj, int head, int count,
                                         int lane, int T, AccFF& acc) {
  const int tm = lane / T, tl = lane - tm * T, nteams = 32 / T;
  for (int e0 = 0; e0 < count; e0 += nteams) {
    const int e = e0 + tm;
    int f = 0, b0 = 0, lenj = 0, actj = 0;
    float3 Do = make_float3(0.f, 0.f, 0.f), Dn = Do, Dol = Do, Dnl = Do;
    if (e < count) {
      const int jf = rj[(head + e) & (kRing - 1)];
      const int j = jf >> 4;
      f = jf & 15;
      float mrj;
      if (!LO && H.uniform) {
        // uniform chain: the neighbour's rows follow from its index
        b0 = H.atom0 + (j - H.mol0) * H.ulen;
        lenj = H.ulen;
        actj = H.uact;
        mrj = H.umrad;
      } else {
        b0 = P.mstart[j];
        const int lw = P.mlen[j];
        lenj = lw & 255;
        actj = lw >> 8;
        mrj = P.mrad[j];
      }
      const uint4 fj = P.mfix[j];
      const float rr = mi.rad + mrj;
      if (f & kInOld) {
        if (PRECISE) fixdiff_ff(fj, mi.fx_old, H, Do, Dol); else Do = fixdiff(fj, mi.fx_old, H);
        if (needs_wrap(Do, rr, H)) f |= kWrapOld;
      }
      if (f & kInNew) {
        if (PRECISE) fixdiff_ff(fj, mi.fx_new, H, Dn, Dnl); else Dn = fixdiff(fj, mi.fx_new, H);
        if (needs_wrap(Dn, rr, H)) f |= kWrapNew;
      }
    }
    float so = 0.f, sn = 0.f, sa = 0.f;
    for (int b = b0 + tl; b < b0 + lenj; b += T) {
      const float4 ob = P.aoff[b];
      const float2 qb = P.aeq[b];
      float4 obl = make_float4(0.f, 0.f, 0.f, 0.f);
      if (LO && PRECISE) obl = P.aofl[b];
      if (f & kInOld) {
        float3 bh = make_float3(Do.x + ob.x, Do.y + ob.y, Do.z + ob.z), bl = Dol;
        if (PRECISE) {
          // two-sum of D + o_b per axis, then the low parts
          const float ex = (Do.x - (bh.x - (bh.x - Do.x))) + (ob.x - (bh.x - Do.x));
          const float ey = (Do.y - (bh.y - (bh.y - Do.y))) + (ob.y - (bh.y - Do.y));
          const float ez = (Do.z - (bh.z - (bh.z - Do.z))) + (ob.z - (bh.z - Do.z));
          bl = make_float3(ex + (Dol.x + obl.x), ey + (Dol.y + obl.y), ez + (Dol.z + obl.z));
        }
        so += (f & kWrapOld)
                  ? sum_moved32_wrap<PRECISE>(s.o_old, s.l_old, s.eq, mi.len, bh, bl, ob.w, qb, H, sa)
                  : sum_moved32_cf<PRECISE>(s.o_old, s.l_old, s.eq, mi.len, false, bh, bl, ob.w, qb,
                                            mi.qm, sa);
      }
      if (f & kInNew) {
        float3 bh = make_float3(Dn.x + ob.x, Dn.y + ob.y, Dn.z + ob.z), bl = Dnl;
        if (PRECISE) {
          const float ex = (Dn.x - (bh.x - (bh.x - Dn.x))) + (ob.x - (bh.x - Dn.x));
          const float ey = (Dn.y - (bh.y - (bh.y - Dn.y))) + (ob.y - (bh.y - Dn.y));
          const float ez = (Dn.z - (bh.z - (bh.z - Dn.z))) + (ob.z - (bh.z - Dn.z));
          bl = make_float3(ex + (Dnl.x + obl.x), ey + (Dnl.y + obl.y), ez + (Dnl.z + obl.z));
        }
        sn += (f & kWrapNew)
                  ? sum_moved32_wrap<PRECISE>(s.o_new, s.l_new, s.eq, mi.len, bh, bl, ob.w, qb, H, sa)
                  : sum_moved32_cf<PRECISE>(s.o_new, s.l_new, s.eq, mi.len, true, bh, bl, ob.w, qb,
                                            mi.qm, sa);
      }
    }
    for (int off = T >> 1; off > 0; off >>= 1) {
      so += __shfl_xor_sync(~0u, so, off);
      sn += __shfl_xor_sync(~0u, sn, off);
      sa += __shfl_xor_sync(~0u, sa, off);
    }
    if (tl == 0 && f) {
      if (f & kInOld) {
        ff_add(acc.oh, acc.ol, so);
        acc.np += (long long)mi.act * actj;
      }
      if (f & kInNew) {
        ff_add(acc.nh, acc.nl, sn);
        acc.np += (long long)mi.act * actj;
      }
      acc.ab += sa;
    }
  }
}

// Asynchronous global -> shared copies (cp.async): the data lands in shared
// memory without passing through registers; each thread waits for its own.
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gsrc) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(d), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;" ::: "memory");
}

// batch_ff with one lane per entry (T = 1) for a uniform chain of molecules
// of at most 4 atoms: the entry's anchor and atom offsets follow from the
// neighbour index, so each lane requests all of them at once with async
// copies into its own shared-memory slot (one round trip to L2 instead of
// one per atom, no registers held), and the pair factors come from the
// chain's per-slot template.  Each placement's sum is batch_ff's bit for bit.
//
// ULEN > 0: molecules of ULEN atoms (the inner atom loop unrolls); ljmask
// bits 4k..4k+3: the LJ terms of neighbour atom k with moved atoms 0..3 that
// are not exactly zero (the same in every lane: the chain is uniform).  Both
// placements run through one copy of the pair code (a rolled loop), which
// keeps the step loop's code small enough for the instruction cache.
template <int ULEN>
__device__ __forceinline__ void batch_u1(const Pool& P, const ChainHdr& H, const GroupSmem& s,
                                         const MovedInfo& mi, const int* rj, int head, int count,
                                         int w, int lane, AccFF& acc, unsigned ljmask) {
  if (lane >= count) return;  // lanes are independent: no shuffles below
  const int jf = rj[(head + lane) & (kRing - 1)];
  const int j = jf >> 4;
  const int f = jf & 15;
  const int lenj = ULEN > 0 ? ULEN : H.ulen;
  const int b0 = H.atom0 + (j - H.mol0) * lenj;
  float4* nb = s.nbuf + (w * 32 + lane) * 5;
  cp_async16(nb + 4, P.mfix + j);
  for (int k = 0; k < lenj; k++) cp_async16(nb + k, P.aoff + b0 + k);
  cp_async_wait_all();
  const uint4 fj = *reinterpret_cast<const uint4*>(nb + 4);
  const float rr = mi.rad + H.umrad;
  const float3 z3 = make_float3(0.f, 0.f, 0.f);
  float sa = 0.f;
#pragma unroll 1
  for (int p = 0; p < 2; p++) {
    if (!(f & (p ? kInNew : kInOld))) continue;
    const float3 D = fixdiff(fj, p ? mi.fx_new : mi.fx_old, H);
    const bool wrap = needs_wrap(D, rr, H);
    const float4* o = p ? s.o_new : s.o_old;
    float sp = 0.f;
#pragma unroll 1
    for (int k = 0; k < lenj; k++) {
      const float4 ob = nb[k];
      const float2 qb = s.teq[k];
      const unsigned lm = (ljmask >> (4 * k)) & 15u;
      const float3 bh = make_float3(D.x + ob.x, D.y + ob.y, D.z + ob.z);
      sp += wrap ? sum_moved32_wrap<false, ULEN>(o, s.l_old, s.eq, mi.len, bh, z3, ob.w, qb, H,
                                                 sa, lm)
                 : sum_moved32_cf<false, ULEN>(o, s.l_old, s.eq, mi.len, p != 0, bh, z3, ob.w, qb,
                                               mi.qm, sa, lm);
    }
    if (p)
      ff_add(acc.nh, acc.nl, sp);
    else
      ff_add(acc.oh, acc.ol, sp);
    acc.np += (long long)mi.act * H.uact;
  }
  acc.ab += sa;
}

// FP64 pair terms from the master rows, the reference's per-pair minimum
// image and dummy-site rule (BruteForceStep.cpp:61-76); sb, eb: the
// neighbour atom's blending factors (blend64), the moved atoms' staged in
// s.sd / s.ed.
__device__ __forceinline__ double sum_moved64(const GroupSmem& s, bool use_new, int len, double xb,
                                              double yb, double zb, double sb, double eb, double qb,
                                              const ChainHdr& H) {
  const double* xs = use_new ? s.nx : s.ox;
  const double* ys = use_new ? s.ny : s.oy;
  const double* zs = use_new ? s.nz : s.oz;
  double acc = 0.0;
  if (sb < 0) return acc;
  for (int i = 0; i < len; i++) {
    const double sa = s.sd[i], ea = s.ed[i];
    if (sa < 0) continue;
    const double dx = make_periodic(xb - xs[i], H.L[0]);
    const double dy = make_periodic(yb - ys[i], H.L[1]);
    const double dz = make_periodic(zb - zs[i], H.L[2]);
    const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    acc += pair64(r2, sa, sb, ea, eb, s.qd[i], qb);
  }
  return acc;
}

__device__ __forceinline__ void batch_f64(const Pool& P, const ChainHdr& H, const GroupSmem& s,
                                          const MovedInfo& mi, const int* rj, int head, int count,
                                          int lane, int T, double& eo, double& en, double& ab,
                                          long long& np) {
  const int tm = lane / T, tl = lane - tm * T, nteams = 32 / T;
  for (int e0 = 0; e0 < count; e0 += nteams) {
    const int e = e0 + tm;
    int f = 0, b0 = 0, lenj = 0, actj = 0;
    if (e < count) {
      const int jf = rj[(head + e) & (kRing - 1)];
      const int j = jf >> 4;
      f = jf & 15;
      b0 = P.mstart[j];
      const int lw = P.mlen[j];
      lenj = lw & 255;
      actj = lw >> 8;
    }
    double so = 0.0, sn = 0.0;
    for (int b = b0 + tl; b < b0 + lenj; b += T) {
      const double xb = P.x[b], yb = P.y[b], zb = P.z[b];
      const double2 bl = P.blend[b];
      const double qb = P.q[b];
      if (f & kInOld) so += sum_moved64(s, false, mi.len, xb, yb, zb, bl.x, bl.y, qb, H);
      if (f & kInNew) sn += sum_moved64(s, true, mi.len, xb, yb, zb, bl.x, bl.y, qb, H);
    }
    for (int off = T >> 1; off > 0; off >>= 1) {
      so += __shfl_xor_sync(~0u, so, off);
      sn += __shfl_xor_sync(~0u, sn, off);
    }
    if (tl == 0 && f) {
      if (f & kInOld) { eo += so; np += (long long)mi.act * actj; }
      if (f & kInNew) { en += sn; np += (long long)mi.act * actj; }
      ab += fabs(so) + fabs(sn);
    }
  }
}

// One warp screens candidates [c_begin, c_end) in warp-strided rounds of 32
// (round r of warp w covers c_begin + (r*nw + w)*32 + lane), appends hits to
// its ring and evaluates them in batches of 32.  FP32 pairs accumulate in
// double-float and are added to the FP64 sums at the end.
template <bool F64>
__device__ inline void warp_eval(const Pool& P, const ChainHdr& H, const GroupSmem& s, const MovedInfo& mi,
                          int c_begin, int c_end, int w, int nw, int lane, int T, double& eo,
                          double& en, double& ab, long long& np) {
  int* rj = s.lj + w * kRing;
  int head = 0, tail = 0;
  const unsigned lt = lanemask_lt();
  AccFF acc = {0.f, 0.f, 0.f, 0.f, 0.f, 0};
  for (int base = c_begin + w * 32; base < c_end; base += nw * 32) {
    const int j = base + lane;
    int f = 0;
    // the FP32 screen with the FP64 re-test inside its guard band gives the
    // FP64 test's in-range set exactly, for FP64 and FP32 pair terms alike
    if (j < c_end && j != mi.mol) f = screen_mixed(P, H, s, mi, j);
    const unsigned bal = __ballot_sync(~0u, f != 0);
    if (f) rj[(tail + __popc(bal & lt)) & (kRing - 1)] = (j << 4) | f;
    tail += __popc(bal);
    if (tail - head >= 32) {
      __syncwarp();
      if (F64)
        batch_f64(P, H, s, mi, rj, head, 32, lane, T, eo, en, ab, np);
      else if (H.precise)
        batch_ff<true, true>(P, H, s, mi, rj, head, 32, lane, T, acc);
      else
        batch_ff<false, true>(P, H, s, mi, rj, head, 32, lane, T, acc);
      head += 32;
      __syncwarp();
    }
  }
  __syncwarp();
  if (tail > head) {
    if (F64)
      batch_f64(P, H, s, mi, rj, head, tail - head, lane, T, eo, en, ab, np);
    else if (H.precise)
      batch_ff<true, true>(P, H, s, mi, rj, head, tail - head, lane, T, acc);
    else
      batch_ff<false, true>(P, H, s, mi, rj, head, tail - head, lane, T, acc);
  }
  __syncwarp();
  if (!F64) {
    eo += (double)acc.oh + (double)acc.ol;
    en += (double)acc.nh + (double)acc.nl;
    ab += (double)acc.ab;
    np += acc.np;
  }
}

// Group-wide deterministic sum of (a, b, d, c): warp shuffles, then every
// thread adds the per-warp values in warp order.  Two calls must be
// separated by a group barrier (the scratch is reused).
__device__ __forceinline__ void group_reduce(const Group& g, const GroupSmem& s, double& a,
                                             double& b, double& d, long long& c, int par = 0) {
  for (int off = 16; off > 0; off >>= 1) {
    a += __shfl_xor_sync(~0u, a, off);
    b += __shfl_xor_sync(~0u, b, off);
    d += __shfl_xor_sync(~0u, d, off);
    c += __shfl_xor_sync(~0u, c, off);
  }
  const int nw = g.nwarps();
  double* red = s.red + par * 3 * nw;   // buffer `par` of two
  long long* redl = s.redl + par * nw;
  if ((g.tid & 31) == 0) {
    red[g.warp()] = a;
    red[nw + g.warp()] = b;
    red[2 * nw + g.warp()] = d;
    redl[g.warp()] = c;
  }
  g.sync();
  a = 0.0;
  b = 0.0;
  d = 0.0;
  c = 0;
  for (int w = 0; w < nw; w++) {
    a += red[w];
    b += red[nw + w];
    d += red[2 * nw + w];
    c += redl[w];
  }
}

// Writes the staged new placement of the moved molecule to the pool
// (master rows and mirrors); lanes of one warp.
__device__ __forceinline__ void commit(const Pool& P, const GroupSmem& s, const MovedInfo& mi,
                                       int lane) {
  for (int i = lane; i < mi.len; i += 32) {
    const int a = mi.atom0 + i;
    P.x[a] = s.nx[i];
    P.y[a] = s.ny[i];
    P.z[a] = s.nz[i];
    P.aoff[a] = s.o_new[i];
    P.aofl[a] = s.l_new[i];
  }
  const int2 pi = P.mpi[mi.mol];
  for (int k = lane; k < mi.npidx; k += 32) P.ppos[pi.x + k] = s.p_new[k];
  if (lane == 0) P.mfix[mi.mol] = mi.fx_new;
}

// Recomputes molecule m's mirrors (offsets, screen positions, fixed-point
// anchor) from its master rows; lanes [lane, nl).
__device__ __forceinline__ void refresh_molecule(const Pool& P, const ChainHdr& H, int m, int lane,
                                                 int nl) {
  const int a0 = P.mstart[m], len = P.mlen[m] & 255;
  const int2 pi = P.mpi[m];
  const int an = P.pidx[pi.x];
  const double ax = P.x[an], ay = P.y[an], az = P.z[an];
  for (int i = lane; i < len; i += nl) {
    const int a = a0 + i;
    const float w = P.aoff[a].w;
    const double vx = P.x[a] - ax, vy = P.y[a] - ay, vz = P.z[a] - az;
    const float4 o = make_float4((float)vx, (float)vy, (float)vz, w);
    P.aoff[a] = o;
    P.aofl[a] = make_float4((float)(vx - (double)o.x), (float)(vy - (double)o.y),
                            (float)(vz - (double)o.z), 0.f);
  }
  for (int k = lane; k < pi.y; k += nl) {
    const int q = P.pidx[pi.x + k];
    P.ppos[pi.x + k] = wrap_pos(P.x[q], P.y[q], P.z[q], H);
  }
  if (lane == 0) P.mfix[m] = fixpos(ax, ay, az, H);
}

}  // namespace mcgpu
