// chain.cuh -- the device-resident chain step: FP32 moves on the fixed-point
// + FP32-offset state (move_f32.cuh), screen and pair batches accumulated in
// double-float, decision in FP32 outside a guard band and in FP64 pairs
// inside it.  FP64 instructions are confined to a handful per step.
#pragma once

#include "kernels.cuh"
#include "move_f32.cuh"

namespace mcgpu {

// FP64 position of a chain atom: anchor (fixed point) + FP32 offset, each
// step rounded once (the CPU mirror computes the same two roundings).
__device__ __forceinline__ double chain_coord(unsigned A, float o, double L) {
  return __dadd_rn(__dmul_rn((double)A, L * 2.3283064365386963e-10), (double)o);
}

__device__ __forceinline__ double3 chain_pos3(uint4 A, float4 o, const ChainHdr& H) {
  return make_double3(chain_coord(A.x, o.x, H.L[0]), chain_coord(A.y, o.y, H.L[1]),
                      chain_coord(A.z, o.z, H.L[2]));
}

// The reference's cutoff test (SimulationStep.cpp:325-326, :332-342,
// :377-385) between FP64 positions.
__device__ __forceinline__ bool in_range_pos64(double3 p1, double3 p2, const ChainHdr& H) {
  const double dx = make_periodic(p2.x - p1.x, H.L[0]);
  const double dy = make_periodic(p2.y - p1.y, H.L[1]);
  const double dz = make_periodic(p2.z - p1.z, H.L[2]);
  const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
  return r2 <= __dmul_rn(H.cutoff, H.cutoff);
}

// Screen position (FP32, wrapped into [0, L)) of an atom at anchor A with
// FP32 offset o.
__device__ __forceinline__ float4 chain_screen_pos(uint4 A, float4 o, const ChainHdr& H) {
  const unsigned x = A.x + (unsigned)fixstep(o.x, H.fxinvf[0]);
  const unsigned y = A.y + (unsigned)fixstep(o.y, H.fxinvf[1]);
  const unsigned z = A.z + (unsigned)fixstep(o.z, H.fxinvf[2]);
  return make_float4(__uint2float_rn(x) * H.fxs[0], __uint2float_rn(y) * H.fxs[1],
                     __uint2float_rn(z) * H.fxs[2], 0.f);
}

// misc[] slots written by stage_chain beyond load_moved's: new quaternion,
// acceptance uniform, "trial placement within skin/2 of the Verlet build"
// flag
enum : int { kMiscQn = 16, kMiscU = 20, kMiscNlTrial = 24 };

// One warp stages the proposed FP32 move `mv` of a chain molecule into
// slot s: old and new offsets (o_old, o_new), pair factors and |o|^2 (eq),
// screen positions of the primaries (p_old, p_new), old and new fixed-point
// anchors, the new quaternion.  No FP64.  It reads the molecule's rows
// only, so a move staged ahead stays valid until a commit of that molecule.
__device__ inline void stage_chain(const Pool& P, const ChainHdr& H, const MoveF& mv,
                                   const StageSlot& s, const float4* pcache, int lane) {
  const int m = H.mol0 + mv.mol;
  int a0, lw;
  int2 pi;
  if (H.uniform) {
    a0 = H.atom0 + mv.mol * H.ulen;
    lw = H.ulen | (H.uact << 8);
    pi = make_int2(H.pidx0 + mv.mol, 1);
  } else {
    a0 = P.mstart[m];
    lw = P.mlen[m];
    pi = P.mpi[m];
  }
  const int len = lw & 255;
  const float4 q4 = P.mq[m];
  const uint4 A = P.mfix[m];
  QuatF q;
  q.w = q4.x; q.x = q4.y; q.y = q4.z; q.z = q4.w;
  const QuatF qn = qnormalise(qmul(mv.qd, q));
  float R[9];
  qmatrix(qn, R);
  // anchor displacement from the vertex: o_v - R' t_v + d
  const float4 ov = P.aoff[a0 + mv.vertex];
  const float4 tv = P.atpl[a0 + mv.vertex];
  const float3 onv = mvec(R, tv.x, tv.y, tv.z);
  const float dlx = __fadd_rn(__fsub_rn(ov.x, onv.x), mv.dx);
  const float dly = __fadd_rn(__fsub_rn(ov.y, onv.y), mv.dy);
  const float dlz = __fadd_rn(__fsub_rn(ov.z, onv.z), mv.dz);
  uint4 An;
  An.x = A.x + (unsigned)fixstep(dlx, H.fxinvf[0]);
  An.y = A.y + (unsigned)fixstep(dly, H.fxinvf[1]);
  An.z = A.z + (unsigned)fixstep(dlz, H.fxinvf[2]);
  An.w = 0u;
  float qsum = 0.f;
  for (int i = lane; i < len; i += 32) {
    const int a = a0 + i;
    const float4 o = P.aoff[a];
    const float4 t = P.atpl[a];
    const float2 qe = P.aeq[a];
    const float3 on = mvec(R, t.x, t.y, t.z);
    s.o_old[i] = o;
    s.o_new[i] = make_float4(on.x, on.y, on.z, o.w);
    s.l_old[i] = make_float4(0.f, 0.f, 0.f, 0.f);  // the chain state's offsets are exact
    s.l_new[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    s.eq[i] = make_float4(qe.x, qe.y, fmaf(o.x, o.x, fmaf(o.y, o.y, o.z * o.z)),
                          fmaf(on.x, on.x, fmaf(on.y, on.y, on.z * on.z)));
    qsum += qe.y;
  }
  for (int off = 16; off > 0; off >>= 1) qsum += __shfl_xor_sync(~0u, qsum, off);
  __syncwarp();
  bool near = true;
  for (int k = lane; k < pi.y; k += 32) {
    const int slot = H.uniform ? H.uprim : P.pidx[pi.x + k] - a0;
    s.pa[k] = slot;
    s.p_old[k] = (k == 0 && pcache) ? pcache[m - H.mol0] : P.ppos[pi.x + k];
    const float4 pn = chain_screen_pos(An, s.o_new[slot], H);
    s.p_new[k] = pn;
    if (H.nl_on) near = near && r2_screen(pn, P.pbuild[pi.x + k], H) <= H.nl_half2;
  }
  near = __all_sync(~0u, near);
  if (lane == 0) {
    s.misc[0] = m; s.misc[1] = a0; s.misc[2] = len; s.misc[3] = pi.y;
    s.misc[4] = lw >> 8; s.misc[5] = 3; s.misc[6] = mv.vertex;
    s.misc[8] = (int)A.x; s.misc[9] = (int)A.y; s.misc[10] = (int)A.z;
    s.misc[12] = (int)An.x; s.misc[13] = (int)An.y; s.misc[14] = (int)An.z;
    s.misc[kMiscQn] = __float_as_int(qn.w); s.misc[kMiscQn + 1] = __float_as_int(qn.x);
    s.misc[kMiscQn + 2] = __float_as_int(qn.y); s.misc[kMiscQn + 3] = __float_as_int(qn.z);
    s.misc[kMiscU] = __float_as_int(mv.u);
    s.misc[kMiscNlTrial] = near ? 1 : 0;
    s.misc[kMiscRad] = __float_as_int(H.uniform ? H.umrad : P.mrad[m]);
    s.misc[kMiscQm] = __float_as_int(qsum);
  }
}

// Screen of candidate j against the staged molecule (both placements):
// FP32 distance of the screen positions, decided outright outside the
// guard band around rc^2 and by the reference's FP64 test inside it.  No
// global load outside the guard band (the positions come from the shared-
// memory cache); the entry's anchor differences are formed in the batch.
__device__ __forceinline__ int screen_chain(const Pool& P, const ChainHdr& H, const GroupSmem& s,
                                            const MovedInfo& mi, int j, float4 q0) {
  const int2 pj = H.simple_prim ? make_int2(H.pidx0 + (j - H.mol0), 1) : P.mpi[j];
  int f = 0;
  for (int k2 = 0; k2 < pj.y; k2++) {
    const float4 q = (k2 == 0) ? q0 : P.ppos[pj.x + k2];
    for (int k1 = 0; k1 < mi.npidx; k1++) {
      const float ro = r2_screen(s.p_old[k1], q, H);
      const float rn = r2_screen(s.p_new[k1], q, H);
      if (!(f & kInOld)) {
        if (ro <= H.cut2_lo) {
          f |= kInOld;
        } else if (ro <= H.cut2_hi) {
          const int p2 = P.pidx[pj.x + k2];
          const double3 a = chain_pos3(mi.fx_old, s.o_old[s.pa[k1]], H);
          const double3 b = chain_pos3(P.mfix[j], P.aoff[p2], H);
          if (in_range_pos64(a, b, H)) f |= kInOld;
        }
      }
      if (!(f & kInNew)) {
        if (rn <= H.cut2_lo) {
          f |= kInNew;
        } else if (rn <= H.cut2_hi) {
          const int p2 = P.pidx[pj.x + k2];
          const double3 a = chain_pos3(mi.fx_new, s.o_new[s.pa[k1]], H);
          const double3 b = chain_pos3(P.mfix[j], P.aoff[p2], H);
          if (in_range_pos64(a, b, H)) f |= kInNew;
        }
      }
    }
  }
  return f;
}

// The single-lane pair batch for the chain's molecule length (inner atom
// loop unrolled for 3-site molecules).
__device__ __forceinline__ void batch_u1_any(const Pool& P, const ChainHdr& H, const GroupSmem& s,
                                             const MovedInfo& mi, const int* rj, int head,
                                             int count, int w, int lane, AccFF& acc) {
  if (H.ulen == 3)
    batch_u1<3>(P, H, s, mi, rj, head, count, w, lane, acc, H.ljmask);
  else
    batch_u1<0>(P, H, s, mi, rj, head, count, w, lane, acc, ~0u);
}

// Bits 4k + i: the LJ term between atoms i and k of a uniform chain's
// molecules (at most 4 atoms) is not exactly zero (sigma and epsilon
// products both nonzero in FP32).  The same for every lane.
__device__ __forceinline__ unsigned uniform_lj_mask(const Pool& P, const ChainHdr& H,
                                                    const float2* teq) {
  unsigned m = 0;
  if (!H.uniform || H.ulen > 4) return ~0u;
  for (int k = 0; k < H.ulen; k++)
    for (int i = 0; i < H.ulen; i++) {
      const float sk = P.aoff[H.atom0 + k].w, si = P.aoff[H.atom0 + i].w;
      if (si * sk != 0.f && teq[i].x * teq[k].x != 0.f) m |= 1u << (4 * k + i);
    }
  return m;
}

// One warp screens chain candidates [c_begin, c_end) -- or, with a Verlet
// list, the molecules cand[c_begin .. c_end) -- in warp-strided rounds of 32
// (screen positions from the shared-memory cache when given) and evaluates
// the in-range ones in batches of 32.
__device__ inline void warp_eval_chain(const Pool& P, const ChainHdr& H, const GroupSmem& s,
                                const MovedInfo& mi, const float4* pcache, int c_begin, int c_end,
                                int w, int nw, int lane, int T, AccFF& acc,
                                const int* cand = nullptr) {
  int* rj = s.lj + w * kRing;
  int head = 0, tail = 0;
  const unsigned lt = lanemask_lt();
  // all molecules: warp w screens blocks of 32 consecutive indices; a list
  // (short, in cell order): warp w takes every nw-th entry, so every warp
  // gets its share of the in-range neighbours
  const int rounds = cand ? (c_end - c_begin + 32 * nw - 1) / (32 * nw) : 0;
  const bool u1 = H.uniform && T == 1 && H.ulen <= 4 && !H.precise;
  for (int it = 0;; it++) {
    int idx;
    if (cand) {
      if (it >= rounds) break;
      idx = c_begin + (it * 32 + lane) * nw + w;
    } else {
      const int base = c_begin + w * 32 + it * nw * 32;
      if (base >= c_end) break;
      idx = base + lane;
    }
    const int j = (cand && idx < c_end) ? cand[idx] : idx;
    int f = 0;
    if (idx < c_end && j != mi.mol) {
      float4 q0;
      if (pcache)
        q0 = pcache[j - H.mol0];
      else if (H.simple_prim)
        q0 = P.ppos[H.pidx0 + (j - H.mol0)];
      else
        q0 = P.ppos[P.mpi[j].x];
      f = screen_chain(P, H, s, mi, j, q0);
    }
    const unsigned bal = __ballot_sync(~0u, f != 0);
    if (f) rj[(tail + __popc(bal & lt)) & (kRing - 1)] = (j << 4) | f;
    tail += __popc(bal);
    if (tail - head >= 32) {
      __syncwarp();
      if (u1)
        batch_u1_any(P, H, s, mi, rj, head, 32, w, lane, acc);
      else if (H.precise)
        batch_ff<true, false>(P, H, s, mi, rj, head, 32, lane, T, acc);
      else
        batch_ff<false, false>(P, H, s, mi, rj, head, 32, lane, T, acc);
      head += 32;
      __syncwarp();
    }
  }
  __syncwarp();
  if (tail > head) {
    if (u1)
      batch_u1_any(P, H, s, mi, rj, head, tail - head, w, lane, acc);
    else if (H.precise)
      batch_ff<true, false>(P, H, s, mi, rj, head, tail - head, lane, T, acc);
    else
      batch_ff<false, false>(P, H, s, mi, rj, head, tail - head, lane, T, acc);
  }
  __syncwarp();
}

// Group-wide deterministic double-float sum: warp butterflies, then every
// thread adds the per-warp values in warp order.
__device__ __forceinline__ void group_reduce_ff(const Group& g, const GroupSmem& s, AccFF& a,
                                                int par = 0) {
  for (int off = 16; off > 0; off >>= 1) {
    const float oh = __shfl_xor_sync(~0u, a.oh, off), ol = __shfl_xor_sync(~0u, a.ol, off);
    const float nh = __shfl_xor_sync(~0u, a.nh, off), nl = __shfl_xor_sync(~0u, a.nl, off);
    ff_add2(a.oh, a.ol, oh, ol);
    ff_add2(a.nh, a.nl, nh, nl);
    a.ab += __shfl_xor_sync(~0u, a.ab, off);
    a.np += __shfl_xor_sync(~0u, a.np, off);
  }
  const int nw = g.nwarps();
  // buffer `par` of two; 5 floats per warp fit the 3 doubles reserved per warp
  float* red = (float*)(s.red + par * 3 * nw);
  long long* redl = s.redl + par * nw;
  if ((g.tid & 31) == 0) {
    red[5 * g.warp() + 0] = a.oh;
    red[5 * g.warp() + 1] = a.ol;
    red[5 * g.warp() + 2] = a.nh;
    red[5 * g.warp() + 3] = a.nl;
    red[5 * g.warp() + 4] = a.ab;
    redl[g.warp()] = a.np;
  }
  g.sync();
  a.oh = a.ol = a.nh = a.nl = a.ab = 0.f;
  a.np = 0;
  for (int w = 0; w < nw; w++) {
    ff_add2(a.oh, a.ol, red[5 * w + 0], red[5 * w + 1]);
    ff_add2(a.nh, a.nl, red[5 * w + 2], red[5 * w + 3]);
    a.ab += red[5 * w + 4];
    a.np += redl[w];
  }
}

// FP64 re-take of a step near the decision threshold: FP64 pair terms
// (pair64, BruteForceStep.cpp:48-79) on the FP64 positions of the chain
// state (anchor + offset).  Warp 0 first writes the moved molecule's old
// and new FP64 coordinates and its FP64 parameters to shared memory; the
// caller synchronises.
__device__ inline void stage_chain_f64(const Pool& P, const ChainHdr& H, const GroupSmem& s,
                                       const MovedInfo& mi, int lane) {
  for (int i = lane; i < mi.len; i += 32) {
    const double2 bl = blend64(P.sig[mi.atom0 + i], P.eps[mi.atom0 + i]);
    s.sd[i] = bl.x;
    s.ed[i] = bl.y;
    s.qd[i] = P.q[mi.atom0 + i];
    const double3 a = chain_pos3(mi.fx_old, s.o_old[i], H);
    const double3 b = chain_pos3(mi.fx_new, s.o_new[i], H);
    s.ox[i] = a.x; s.oy[i] = a.y; s.oz[i] = a.z;
    s.nx[i] = b.x; s.ny[i] = b.y; s.nz[i] = b.z;
  }
}

__device__ __forceinline__ void batch_chain64(const Pool& P, const ChainHdr& H, const GroupSmem& s,
                                              const MovedInfo& mi, const int* rj, int head,
                                              int count, int lane, int T, double& eo, double& en) {
  const int tm = lane / T, tl = lane - tm * T, nteams = 32 / T;
  for (int e0 = 0; e0 < count; e0 += nteams) {
    const int e = e0 + tm;
    int f = 0, b0 = 0, lenj = 0;
    uint4 Aj = make_uint4(0u, 0u, 0u, 0u);
    if (e < count) {
      const int jf = rj[(head + e) & (kRing - 1)];
      const int j = jf >> 4;
      f = jf & 15;
      b0 = P.mstart[j];
      lenj = P.mlen[j] & 255;
      Aj = P.mfix[j];
    }
    double so = 0.0, sn = 0.0;
    for (int b = b0 + tl; b < b0 + lenj; b += T) {
      const double3 xb = chain_pos3(Aj, P.aoff[b], H);
      const double2 bl = P.blend ? P.blend[b] : blend64(P.sig[b], P.eps[b]);
      const double sb = bl.x, eb = bl.y, qb = P.q[b];
      if (f & kInOld) so += sum_moved64(s, false, mi.len, xb.x, xb.y, xb.z, sb, eb, qb, H);
      if (f & kInNew) sn += sum_moved64(s, true, mi.len, xb.x, xb.y, xb.z, sb, eb, qb, H);
    }
    for (int off = T >> 1; off > 0; off >>= 1) {
      so += __shfl_xor_sync(~0u, so, off);
      sn += __shfl_xor_sync(~0u, sn, off);
    }
    if (tl == 0 && f) {
      if (f & kInOld) eo += so;
      if (f & kInNew) en += sn;
    }
  }
}

// The FP64 re-take's screen: the reference's test for every primary pair
// on the chain state's FP64 positions.
//
// With a Verlet list (cand non-null), the molecules cand[c_begin .. c_end),
// every nw-th entry per warp as in warp_eval_chain.
__device__ inline void warp_eval_chain64(const Pool& P, const ChainHdr& H, const GroupSmem& s,
                                  const MovedInfo& mi, const float4* pcache, int c_begin,
                                  int c_end, int w, int nw, int lane, int T, double& eo,
                                  double& en, const int* cand = nullptr) {
  int* rj = s.lj + w * kRing;
  int head = 0, tail = 0;
  const unsigned lt = lanemask_lt();
  const int rounds = cand ? (c_end - c_begin + 32 * nw - 1) / (32 * nw) : 0;
  for (int it = 0;; it++) {
    int idx;
    if (cand) {
      if (it >= rounds) break;
      idx = c_begin + (it * 32 + lane) * nw + w;
    } else {
      const int base = c_begin + w * 32 + it * nw * 32;
      if (base >= c_end) break;
      idx = base + lane;
    }
    const int j = (cand && idx < c_end) ? cand[idx] : idx;
    int f = 0;
    // the step's own screen: FP32 outside the guard band, the FP64 test on
    // these same FP64 positions inside it -- the FP64 in-range set exactly,
    // without an FP64 distance for every candidate
    if (idx < c_end && j != mi.mol) {
      float4 q0;
      if (pcache)
        q0 = pcache[j - H.mol0];
      else if (H.simple_prim)
        q0 = P.ppos[H.pidx0 + (j - H.mol0)];
      else
        q0 = P.ppos[P.mpi[j].x];
      f = screen_chain(P, H, s, mi, j, q0);
    }
  const unsigned bal = __ballot_sync(~0u, f != 0);
    if (f) rj[(tail + __popc(bal & lt)) & (kRing - 1)] = (j << 4) | f;
    tail += __popc(bal);
    if (tail - head >= 32) {
      __syncwarp();
      batch_chain64(P, H, s, mi, rj, head, 32, lane, T, eo, en);
      head += 32;
      __syncwarp();
    }
  }
  __syncwarp();
  if (tail > head) batch_chain64(P, H, s, mi, rj, head, tail - head, lane, T, eo, en);
  __syncwarp();
}

// Commit of an accepted chain move: offsets, quaternion, anchor, screen
// positions (and the shared-memory screen cache).
__device__ __forceinline__ void commit_chain(const Pool& P, const ChainHdr& H, const GroupSmem& s,
                                             const MovedInfo& mi, float4* pcache, int lane) {
  for (int i = lane; i < mi.len; i += 32) P.aoff[mi.atom0 + i] = s.o_new[i];
  const int2 pi = H.uniform ? make_int2(H.pidx0 + (mi.mol - H.mol0), 1) : P.mpi[mi.mol];
  for (int k = lane; k < mi.npidx; k += 32) P.ppos[pi.x + k] = s.p_new[k];
  if (lane == 0) {
    P.mfix[mi.mol] = mi.fx_new;
    P.mq[mi.mol] = make_float4(__int_as_float(s.misc[kMiscQn]), __int_as_float(s.misc[kMiscQn + 1]),
                               __int_as_float(s.misc[kMiscQn + 2]),
                               __int_as_float(s.misc[kMiscQn + 3]));
    if (pcache) pcache[mi.mol - H.mol0] = s.p_new[0];
  }
}

}  // namespace mcgpu
