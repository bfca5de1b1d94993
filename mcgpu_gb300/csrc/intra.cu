// intra.cu -- flexible molecules on the plain path: the reference's
// intramolecular energy, bond stretch and angle expansion
// (src/Metropolis/SimulationStep.cpp:80-315), which it compiles but calls
// only with ENABLE_INTRA true (SimulationStep.h:15).
//
// A stage is one CTA on one molecule (a molecule has at most 64 atoms): the
// ops of the stage run in order, each as a scalar set-up by thread 0 (the
// bond's unit vector or the plane normal) and one update per atom; then the
// molecule's mirrors and radius, and the intramolecular energy.  The union-
// find the reference runs on every call depends only on the bonds, so its
// partitions are computed once on the host at upload.  Coordinates follow
// the reference's FP64 operations one for one with explicit round-to-nearest
// intrinsics (no contraction) and the host's C-library cosines and sines, so
// they are the reference's bit for bit; the energies are FP64 sums in a
// different order (equal to the reference's within FP64 rounding).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "intra.h"
#include "kernels.cuh"

namespace mcgpu {

namespace {

constexpr int kIntraThreads = 128;

// The SimCalcs pair terms of the intramolecular energy (SimulationStep.cpp:
// 344-375): blending by sqrt|a b| (sites with negative sigma or epsilon take
// part), no cutoff, zero at r = 0.  1/r from one FP64 rsqrt (a few ulps from
// the reference's sqrt and divisions, which cost many FP64 passes on this
// part); sigma^2 = |s_i s_j| and 4 eps = 4 sqrt|e_i e_j|.
__device__ __forceinline__ double intra_pair(const Pool& P, int i, int j, const ChainHdr& H) {
  const double dx = make_periodic(__dsub_rn(P.x[j], P.x[i]), H.L[0]);
  const double dy = make_periodic(__dsub_rn(P.y[j], P.y[i]), H.L[1]);
  const double dz = make_periodic(__dsub_rn(P.z[j], P.z[i]), H.L[2]);
  const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
  if (r2 == 0.0) return 0.0;
  const double ri = rsqrt(r2);
  const double ss = fabs(P.sig[i] * P.sig[j]);
  const double ee = P.eps[i] * P.eps[j];
  const double s2 = ss * (ri * ri);
  const double s6 = s2 * s2 * s2;
  const double lj = 4.0 * sqrt(fabs(ee)) * (s6 * s6 - s6);
  return lj + P.q[i] * P.q[j] * 332.06 * ri;
}

// Block-wide deterministic sum of three values (every thread gets them).
__device__ __forceinline__ void block_sum3(double& a, double& b, double& c, double* red) {
  for (int off = 16; off > 0; off >>= 1) {
    a += __shfl_xor_sync(~0u, a, off);
    b += __shfl_xor_sync(~0u, b, off);
    c += __shfl_xor_sync(~0u, c, off);
  }
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) {
    red[w] = a;
    red[nw + w] = b;
    red[2 * nw + w] = c;
  }
  __syncthreads();
  a = b = c = 0.0;
  for (int k = 0; k < nw; k++) {
    a += red[k];
    b += red[nw + k];
    c += red[2 * nw + k];
  }
}

// SimCalcs::calcIntraMolecularEnergy (SimulationStep.cpp:80-129) of box
// molecule mol (pool molecule m), all threads of the block.
__device__ double intra_energy(const Pool& P, const IntraRows& R, const ChainHdr& H, int mol,
                               double* red) {
  const int m = H.mol0 + mol;
  const int tid = threadIdx.x, nt = blockDim.x;
  double ea = 0.0, eb = 0.0, ep = 0.0;
  if (R.flex_angles) {
    const int s = R.m_astart[mol], e = s + R.m_acount[mol];
    for (int k = s + tid; k < e; k += nt)
      if (R.a_var[k]) {
        const double d = R.a_eq[k] - R.a_size[k];
        ea += R.a_k[k] * d * d;
      }
  }
  if (R.flex_bonds) {
    const int s = R.m_bstart[mol], e = s + R.m_bcount[mol];
    for (int k = s + tid; k < e; k += nt)
      if (R.b_var[k]) {
        const double d = R.b_eq[k] - R.b_len[k];
        eb += R.b_k[k] * d * d;
      }
  }
  if (R.flex_bonds || R.flex_angles) {
    const int a0 = P.mstart[m], len = P.mlen[m] & 255;
    const int ty = R.m_type[mol], n = R.t_natom[ty];
    const unsigned char* code = R.code + R.t_off[ty];
    for (int q = tid; q < len * len; q += nt) {
      const int i = q / len, j = q - i * len;
      if (j <= i) continue;
      const int c = (i < n && j < n) ? code[i * n + j] : 2;
      if (c == 0) continue;
      const double e = intra_pair(P, a0 + i, a0 + j, H);
      ep += c == 1 ? 0.5 * e : e;
    }
  }
  block_sum3(ea, eb, ep, red);
  double out = 0.0;
  if (R.flex_angles) out += ea;
  if (R.flex_bonds) out += eb;
  return out + ep;
}

// The molecule's mirrors after its atoms moved, and its radius (max
// distance of an atom from the first primary atom, with the margin the
// upload gives it): the FP32 pair paths decide per-pair images from it.
__device__ void refresh_flexible(const Pool& P, const ChainHdr& H, int m, double* red) {
  refresh_molecule(P, H, m, threadIdx.x, blockDim.x);
  const int a0 = P.mstart[m], len = P.mlen[m] & 255;
  const int an = P.pidx[P.mpi[m].x];
  double r = 0.0;
  for (int i = threadIdx.x; i < len; i += blockDim.x) {
    const double dx = P.x[a0 + i] - P.x[an], dy = P.y[a0 + i] - P.y[an],
                 dz = P.z[a0 + i] - P.z[an];
    r = fmax(r, sqrt(dx * dx + dy * dy + dz * dz));
  }
  for (int off = 16; off > 0; off >>= 1) r = fmax(r, __shfl_xor_sync(~0u, r, off));
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[w] = r;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 0; k < nw; k++) r = fmax(r, red[k]);
    P.mrad[m] = (float)(r * (1 + 1e-6) + 1e-4);
  }
}

__global__ void __launch_bounds__(kIntraThreads) k_intra_energy(Pool P, IntraRows R, int chain,
                                                                int mol, double* out) {
  __shared__ double red[3 * (kIntraThreads / 32)];
  const ChainHdr& H = P.hdr[chain];
  const double e = intra_energy(P, R, H, mol, red);
  if (threadIdx.x == 0) out[0] = e;
}

__global__ void __launch_bounds__(kIntraThreads) k_intra_add(Pool P, IntraRows R, double* emol) {
  __shared__ double red[3 * (kIntraThreads / 32)];
  const ChainHdr& H = P.hdr[0];
  const int mol = blockIdx.x;
  const double e = intra_energy(P, R, H, mol, red);
  if (threadIdx.x == 0) emol[H.mol0 + mol] += e;
}

// One SimCalcs::stretchBond (kind 0, SimulationStep.cpp:257-315) or
// SimCalcs::expandAngle (kind 1, :148-239) of entry i of box molecule mol,
// every thread of the block; c1, s1 / c2, s2: the cosine and sine of the
// first / second group's angle.  Returns false when the call changes nothing
// (a bond in a ring, an angle whose ends share a component).
__device__ bool apply_op(const Pool& P, const IntraRows& R, const ChainHdr& H, int mol, int kind,
                         int i, double amt, double c1, double s1, double c2, double s2,
                         double* sv) {
  const int m = H.mol0 + mol;
  const int a0 = P.mstart[m], len = P.mlen[m] & 255;
  const int tid = threadIdx.x;
  if (kind == 0) {
    const int b = R.m_bstart[mol] + i;
    const int off = R.b_part[b];
    if (off < 0) return false;  // a ring: the reference returns before moving
    if (tid < 3) {
      // lanes 0-2 each form the whole vector and its length (same values)
      // and divide their own component: one division's latency, not three.
      // (v / d) / 2 == (v / d) * 0.5 exactly.
      const int e1 = H.atom0 + R.b_a1[b], e2 = H.atom0 + R.b_a2[b];
      const double vx = __dsub_rn(P.x[e2], P.x[e1]);
      const double vy = __dsub_rn(P.y[e2], P.y[e1]);
      const double vz = __dsub_rn(P.z[e2], P.z[e1]);
      double d = __dadd_rn(0.0, __dmul_rn(vx, vx));
      d = __dadd_rn(d, __dmul_rn(vy, vy));
      d = __dadd_rn(d, __dmul_rn(vz, vz));
      d = __dsqrt_rn(d);
      const double vc = tid == 0 ? vx : (tid == 1 ? vy : vz);
      sv[tid] = __dmul_rn(__ddiv_rn(vc, d), 0.5);
      if (tid == 0) R.b_len[b] = __dadd_rn(R.b_len[b], amt);
    }
    __syncthreads();
    if (tid < len) {
      const int a = a0 + tid;
      const double sx = __dmul_rn(sv[0], amt), sy = __dmul_rn(sv[1], amt),
                   sz = __dmul_rn(sv[2], amt);
      if (R.part[off + tid] == 1) {
        P.x[a] = __dadd_rn(P.x[a], sx);
        P.y[a] = __dadd_rn(P.y[a], sy);
        P.z[a] = __dadd_rn(P.z[a], sz);
      } else {
        P.x[a] = __dsub_rn(P.x[a], sx);
        P.y[a] = __dsub_rn(P.y[a], sy);
        P.z[a] = __dsub_rn(P.z[a], sz);
      }
    }
    __syncthreads();
    return true;
  }
  const int g = R.m_astart[mol] + i;
  const int off = R.a_part[g];
  if (off < 0) return false;  // both ends in one component
  if (tid < 3) {
    // lanes 0-2: the same normal and length, one component's division each
    const int e1 = H.atom0 + R.a_a1[g], e2 = H.atom0 + R.a_a2[g], md = H.atom0 + R.a_mid[g];
    const double m0 = P.x[md], m1 = P.y[md], m2 = P.z[md];
    const double p0 = __dsub_rn(m0, P.x[e1]), p1 = __dsub_rn(m1, P.y[e1]),
                 p2 = __dsub_rn(m2, P.z[e1]);
    const double q0 = __dsub_rn(m0, P.x[e2]), q1 = __dsub_rn(m1, P.y[e2]),
                 q2 = __dsub_rn(m2, P.z[e2]);
    const double n0 = __dsub_rn(__dmul_rn(p1, q2), __dmul_rn(q1, p2));
    const double n1 = __dsub_rn(__dmul_rn(q0, p2), __dmul_rn(p0, q2));
    const double n2 = __dsub_rn(__dmul_rn(p0, q1), __dmul_rn(q0, p1));
    double nl = __dadd_rn(0.0, __dmul_rn(n0, n0));
    nl = __dadd_rn(nl, __dmul_rn(n1, n1));
    nl = __dadd_rn(nl, __dmul_rn(n2, n2));
    nl = __dsqrt_rn(nl);
    const double nc = tid == 0 ? n0 : (tid == 1 ? n1 : n2);
    sv[tid] = __ddiv_rn(nc, nl);
    sv[3 + tid] = tid == 0 ? m0 : (tid == 1 ? m1 : m2);
    if (tid == 0) R.a_size[g] = __dadd_rn(R.a_size[g], amt);
  }
  __syncthreads();
  if (tid < len) {
    const int lab = R.part[off + tid];
    if (lab) {
      const double cs = lab == 1 ? c1 : c2;
      const double sn = lab == 1 ? s1 : s2;
      const double omc = __dsub_rn(1.0, cs);
      const int a = a0 + tid;
      const double t0 = __dsub_rn(P.x[a], sv[3]), t1 = __dsub_rn(P.y[a], sv[4]),
                   t2 = __dsub_rn(P.z[a], sv[5]);
      double dot = __dadd_rn(0.0, __dmul_rn(t0, sv[0]));
      dot = __dadd_rn(dot, __dmul_rn(t1, sv[1]));
      dot = __dadd_rn(dot, __dmul_rn(t2, sv[2]));
      const double k0 = __dsub_rn(__dmul_rn(sv[1], t2), __dmul_rn(t1, sv[2]));
      const double k1 = __dsub_rn(__dmul_rn(t0, sv[2]), __dmul_rn(sv[0], t2));
      const double k2 = __dsub_rn(__dmul_rn(sv[0], t1), __dmul_rn(t0, sv[1]));
      const double u0 = __dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(sv[0], dot), omc),
                                            __dmul_rn(t0, cs)), __dmul_rn(k0, sn));
      const double u1 = __dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(sv[1], dot), omc),
                                            __dmul_rn(t1, cs)), __dmul_rn(k1, sn));
      const double u2 = __dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(sv[2], dot), omc),
                                            __dmul_rn(t2, cs)), __dmul_rn(k2, sn));
      P.x[a] = __dadd_rn(u0, sv[3]);
      P.y[a] = __dadd_rn(u1, sv[4]);
      P.z[a] = __dadd_rn(u2, sv[5]);
    }
  }
  __syncthreads();
  return true;
}

// SimCalcs::saveBonds / saveAngles (SimulationStep.cpp:678-701), all threads.
__device__ void save_rows(const IntraRows& R, int mol) {
  for (int k = R.m_bstart[mol] + threadIdx.x; k < R.m_bstart[mol] + R.m_bcount[mol];
       k += blockDim.x)
    R.b_len_rb[k] = R.b_len[k];
  for (int k = R.m_astart[mol] + threadIdx.x; k < R.m_astart[mol] + R.m_acount[mol];
       k += blockDim.x)
    R.a_size_rb[k] = R.a_size[k];
}

// Rollback with the ENABLE_INTRA branch (SimulationStep.cpp:731-775):
// coordinates from the rollback copy, angle sizes and bond lengths from
// theirs, then the mirrors; all threads.
__device__ void rollback_rows(const Pool& P, const IntraRows& R, const ChainHdr& H, int chain,
                              int mol, double* red) {
  const int m = H.mol0 + mol;
  const int a0 = P.mstart[m], len = P.mlen[m] & 255;
  const double* rb = P.rb + (size_t)chain * 3 * H.max_len;
  for (int i = threadIdx.x; i < len; i += blockDim.x) {
    P.x[a0 + i] = rb[i];
    P.y[a0 + i] = rb[H.max_len + i];
    P.z[a0 + i] = rb[2 * H.max_len + i];
  }
  for (int k = R.m_astart[mol] + threadIdx.x; k < R.m_astart[mol] + R.m_acount[mol];
       k += blockDim.x)
    R.a_size[k] = R.a_size_rb[k];
  for (int k = R.m_bstart[mol] + threadIdx.x; k < R.m_bstart[mol] + R.m_bcount[mol];
       k += blockDim.x)
    R.b_len[k] = R.b_len_rb[k];
  __syncthreads();
  refresh_flexible(P, H, m, red);
}

__global__ void __launch_bounds__(kIntraThreads) k_intra_ops(Pool P, IntraRows R, int chain,
                                                             IntraOps ops, double* out) {
  __shared__ double red[3 * (kIntraThreads / 32)];
  __shared__ double sv[9];
  const ChainHdr& H = P.hdr[chain];
  const int mol = ops.mol, m = H.mol0 + mol;
  const int tid = threadIdx.x;
  if (ops.flags & kIntraSave) save_rows(R, mol);
  __syncthreads();
  if (ops.flags & kIntraEnergyBefore) {
    const double e = intra_energy(P, R, H, mol, red);
    if (tid == 0) out[0] = e;
  }
  bool moved = false;
  for (int k = 0; k < ops.n; k++)
    moved |= apply_op(P, R, H, mol, ops.kind, ops.idx[k], ops.amt[k], ops.c1[k], ops.s1[k],
                      ops.c2[k], ops.s2[k], sv);
  if (moved) {
    refresh_flexible(P, H, m, red);
    __syncthreads();
  }
  if (ops.flags & kIntraEnergyAfter) {
    const double e = intra_energy(P, R, H, mol, red);
    if (tid == 0) out[1] = e;
  }
}

__global__ void __launch_bounds__(kIntraThreads) k_intra_rollback(Pool P, IntraRows R, int chain,
                                                                  int mol) {
  __shared__ double red[3 * (kIntraThreads / 32)];
  rollback_rows(P, R, P.hdr[chain], chain, mol, red);
}

// ---- the reference's loop on the device ----------------------------------------

constexpr int kLoopThreads = 256;
constexpr int kLoopDrawCap = 1 << 20;

// randomReal (MathLibrary.cpp:31-33) on the restated C-library stream,
// operation by operation.
__device__ __forceinline__ double loop_real(CRand& g, double start, double end) {
  const double r = __ddiv_rn((double)crand_next(g), 2147483647.0);
  return __dadd_rn(__dmul_rn(__dsub_rn(end, start), r), start);
}

// acceptMove (SimulationStep.cpp:794-803): no draw for a decrease.
__device__ __forceinline__ bool loop_accept(CRand& g, double de, double kT) {
  if (de < 0) return true;
  return exp(-(de) / kT) >= loop_real(g, 0.0, 1.0);
}

// Thread 0: the draws of one stage of intramolecularMove (kind 0 bonds,
// :589-609; kind 1 angles, :621-640): how many, which (a std::set's distinct
// draws in ascending order), an amount each; the variable entries go to
// sel / amt.  Returns the count the counters take, or -1 when the set did
// not fill within the draw cap.
__device__ int loop_draw_stage(CRand& g, const IntraRows& R, int mol, int kind, double delta,
                               int max_moves, int* sel, double* amt, int* n_sel) {
  const int count = kind == 0 ? R.m_bcount[mol] : R.m_acount[mol];
  const int start = kind == 0 ? R.m_bstart[mol] : R.m_astart[mol];
  const int* var = kind == 0 ? R.b_var : R.a_var;
  int n = count;
  if (n > 3) n = min((int)loop_real(g, 2, count), max_moves);
  // 0.25 + (0.75 / n) * intraScaleFactor, rounded step by step as the host does
  const double scale = __dadd_rn(0.25, __dmul_rn(__ddiv_rn(0.75, (double)n), 0.625));
  int have = 0, draws = 0;
  while (have < n) {
    if (++draws > kLoopDrawCap) return -1;
    const int v = min((int)loop_real(g, 0, count), count - 1);
    int pos = 0;
    while (pos < have && sel[pos] < v) pos++;
    if (pos < have && sel[pos] == v) continue;
    for (int k = have; k > pos; k--) sel[k] = sel[k - 1];
    sel[pos] = v;
    have++;
  }
  int ns = 0;
  for (int k = 0; k < have; k++) {
    const double d = __dmul_rn(scale, loop_real(g, -delta, delta));
    if (var[start + sel[k]]) {
      sel[ns] = sel[k];
      amt[ns] = d;
      ns++;
    }
  }
  *n_sel = ns;
  return n;
}

template <bool F64>
__global__ void __launch_bounds__(kLoopThreads) k_plain_steps(const LoopTask* tasks, int n_steps,
                                                              SmemShape shape) {
  extern __shared__ __align__(16) char smem[];
  __shared__ LoopTask task;
  if (threadIdx.x == 0) task = tasks[blockIdx.x];
  __syncthreads();
  const Pool& P = task.P;
  const IntraRows& R = task.R;
  const int intra = task.intra;
  PlainLoop* L = task.L;
  __shared__ PlainLoop st;
  __shared__ Proposal prop;
  __shared__ double red[3 * (kLoopThreads / 32)];
  __shared__ double sv[9];
  __shared__ int sel[kLoopSel];
  __shared__ double amt[kLoopSel], trig[4 * kLoopSel];
  __shared__ int n_sel, flag, stop;
  const ChainHdr& H = P.hdr[0];
  Group grp{(int)threadIdx.x, (int)blockDim.x, 1};
  GroupSmem s = shape.carve(smem);
  const int tid = threadIdx.x, lane = tid & 31, w = grp.warp(), nw = grp.nwarps();
  const int n = H.n_mol;
  const double kT = H.kT, max_t = H.max_t, max_r = H.max_r;
  const double deg2rad = 3.14159256358979323846264 / 180.0;   // expandAngle's constant
  if (tid == 0) {
    st = *L;
    stop = 0;
  }
  __syncthreads();
  for (int k = 0; k < n_steps; k++) {
    if (tid == 0) {
      // chooseMolecule and the seven intermolecularMove draws
      // (SimulationStep.cpp:25-27, 527-535), clamped as the host loop clamps
      CRand& g = st.rng;
      const int mol = min((int)loop_real(g, 0, n), n - 1);
      const int len = P.mlen[H.mol0 + mol] & 255;
      memset(&prop, 0, sizeof(prop));
      prop.mol = mol;
      prop.mode = MCGPU_ROT_EULER;
      prop.vertex = min((int)loop_real(g, 0, len), len - 1);
      prop.dx = loop_real(g, -max_t, max_t);
      prop.dy = loop_real(g, -max_t, max_t);
      prop.dz = loop_real(g, -max_t, max_t);
      prop.r0 = loop_real(g, -max_r, max_r);
      prop.r1 = loop_real(g, -max_r, max_r);
      prop.r2 = loop_real(g, -max_r, max_r);
    }
    __syncthreads();
    const int mol = prop.mol, m = H.mol0 + mol;
    double eo = 0.0, en = 0.0, ab = 0.0;
    long long np = 0;
    if (!intra) {
      // old and new placement in one pass (k_move_energies on one CTA)
      if (w == 0) stage(P, H, m, &prop, s, lane);
      grp.sync();
      const MovedInfo mi = load_moved(s);
      warp_eval<F64>(P, H, s, mi, H.mol0, H.mol0 + n, w, nw, lane, H.tpm, eo, en, ab, np);
      group_reduce(grp, s, eo, en, ab, np);
      if (tid == 0) {
        const double de = en - eo;
        flag = loop_accept(st.rng, de, kT);
        st.pairs += np;
        if (flag) {
          st.energy += de;
          st.accepted++;
        } else {
          st.rejected++;
        }
      }
      __syncthreads();
      if (flag && w == 0) commit(P, s, mi, lane);
      __syncthreads();
      continue;
    }
    // ---- with the intramolecular term and move ----
    const double ei_old = intra_energy(P, R, H, mol, red);
    if (w == 0) stage(P, H, m, nullptr, s, lane);
    grp.sync();
    {
      const MovedInfo mi = load_moved(s);
      warp_eval<F64>(P, H, s, mi, H.mol0, H.mol0 + n, w, nw, lane, H.tpm, eo, en, ab, np);
      group_reduce(grp, s, eo, en, ab, np);
    }
    const double e_old = eo + ei_old;
    long long pairs = np;
    __syncthreads();
    // the rigid move: rollback copy, move, wrap, commit
    if (w == 0) {
      stage(P, H, m, &prop, s, lane);
      __syncwarp();
      const MovedInfo mi = load_moved(s);
      double* rb = P.rb;
      for (int i = lane; i < mi.len; i += 32) {
        rb[i] = s.ox[i];
        rb[H.max_len + i] = s.oy[i];
        rb[2 * H.max_len + i] = s.oz[i];
      }
      commit(P, s, mi, lane);
    }
    __syncthreads();
    // SimCalcs::intramolecularMove (SimulationStep.cpp:568-675)
    save_rows(R, mol);
    const double bond_delta = st.max_bond_delta, angle_delta = st.max_angle_delta;
    __syncthreads();
    double cur = 0.0;
    bool have_cur = false;
    for (int kind = 0; kind < 2; kind++) {
      if (kind == 0 ? !R.flex_bonds : !R.flex_angles) continue;
      if (tid == 0) {
        const int cnt = loop_draw_stage(st.rng, R, mol, kind, kind == 0 ? bond_delta : angle_delta,
                                        st.max_intra_moves, sel, amt, &n_sel);
        if (cnt < 0) {
          st.error = 1;
          stop = 1;
        } else if (kind == 0) {
          st.bond_moves += cnt;
        } else {
          st.angle_moves += cnt;
        }
        flag = cnt;
        for (int q = 0; kind == 1 && q < n_sel; q++) {
          sincos(__dmul_rn(amt[q], -deg2rad), &trig[4 * q + 1], &trig[4 * q]);
          sincos(__dmul_rn(amt[q], deg2rad), &trig[4 * q + 3], &trig[4 * q + 2]);
        }
      }
      __syncthreads();
      if (stop) break;
      const int cnt = flag;
      const double e0 = have_cur ? cur : intra_energy(P, R, H, mol, red);
      bool moved = false;
      for (int q = 0; q < n_sel; q++)
        moved |= apply_op(P, R, H, mol, kind, sel[q], amt[q], trig[4 * q], trig[4 * q + 1],
                          trig[4 * q + 2], trig[4 * q + 3], sv);
      if (moved) {
        refresh_flexible(P, H, m, red);
        __syncthreads();
      }
      const double e1 = intra_energy(P, R, H, mol, red);
      if (tid == 0 && loop_accept(st.rng, e1 - e0, kT)) {
        if (kind == 0)
          st.bond_accepted += cnt;
        else
          st.angle_accepted += cnt;
      }
      cur = e1;
      have_cur = true;
      __syncthreads();
    }
    if (stop) break;
    if (tid == 0 && st.step != 0 && (st.step % 1000) == 0) {
      // width tuning (:656-674); the angle test reads the entry width
      const double bond_ratio = (double)st.bond_accepted / st.bond_moves;
      const double angle_ratio = (double)st.angle_accepted / st.angle_moves;
      double diff = bond_ratio - 0.4;
      if (fabs(diff) > 0.0001)
        st.max_bond_delta = __dadd_rn(st.max_bond_delta, __dmul_rn(st.max_bond_delta, diff));
      diff = angle_ratio - 0.4;
      if (fabs(angle_delta) > 0.0001)
        st.max_angle_delta = __dadd_rn(st.max_angle_delta, __dmul_rn(st.max_angle_delta, diff));
      st.bond_accepted = st.bond_moves = 0;
      st.angle_accepted = st.angle_moves = 0;
    }
    // the new energy: the intramolecular part is the last stage's (the same
    // coordinates and rows), else computed here
    const double ei_new = have_cur ? cur : intra_energy(P, R, H, mol, red);
    if (w == 0) stage(P, H, m, nullptr, s, lane);
    grp.sync();
    eo = en = ab = 0.0;
    np = 0;
    {
      const MovedInfo mi = load_moved(s);
      warp_eval<F64>(P, H, s, mi, H.mol0, H.mol0 + n, w, nw, lane, H.tpm, eo, en, ab, np);
      group_reduce(grp, s, eo, en, ab, np);
    }
    if (tid == 0) {
      const double de = (eo + ei_new) - e_old;
      flag = loop_accept(st.rng, de, kT);
      st.pairs += pairs + np;
      if (flag) {
        st.energy += de;
        st.accepted++;
      } else {
        st.rejected++;
      }
      st.step++;
    }
    __syncthreads();
    if (!flag) rollback_rows(P, R, H, 0, mol, red);
    __syncthreads();
  }
  if (tid == 0) *L = st;
}

// Union-find over local atom indexes (the partition is all that is used).
int uf_find(std::vector<int>& p, int a) {
  while (p[a] != a) {
    p[a] = p[p[a]];
    a = p[a];
  }
  return a;
}

}  // namespace

IntraHost::~IntraHost() {
  for (void* p : allocs)
    if (p) cudaFree(p);
  if (hout) cudaFreeHost(hout);
}

int intra_upload(mcgpu_ctx* ctx, int n_mol, int n_atom, const int* mol_start, const int* mol_len,
                 const mcgpu_topology_desc* t, std::unique_ptr<IntraHost>* out) {
  if (!t) return set_err(ctx, MCGPU_ERR_INVALID, "null topology");
  const int nb = t->n_bond, na = t->n_angle, nt = t->n_type;
  if (nb < 0 || na < 0 || nt < 0) return set_err(ctx, MCGPU_ERR_INVALID, "negative topology size");
  if ((nb && (!t->bond_a1 || !t->bond_a2 || !t->bond_var || !t->bond_k || !t->bond_eq ||
              !t->bond_len)) ||
      (na && (!t->angle_a1 || !t->angle_a2 || !t->angle_mid || !t->angle_var || !t->angle_k ||
              !t->angle_eq || !t->angle_size)) ||
      !t->mol_bond_start || !t->mol_bond_count || !t->mol_angle_start || !t->mol_angle_count ||
      !t->mol_type || (nt && !t->type_natom))
    return set_err(ctx, MCGPU_ERR_INVALID, "null topology row");
  if (t->max_intra_moves < 0)
    return set_err(ctx, MCGPU_ERR_INVALID, "negative max_intra_moves");
  std::vector<int> t_off(std::max(nt, 1), 0);
  long long codes = 0;
  for (int k = 0; k < nt; k++) {
    if (t->type_natom[k] < 0 || t->type_natom[k] > MCGPU_MAX_MOL_ATOMS)
      return set_err(ctx, MCGPU_ERR_INVALID, "type %d: %d atoms", k, t->type_natom[k]);
    t_off[k] = (int)codes;
    codes += (long long)t->type_natom[k] * t->type_natom[k];
  }
  if (codes && !t->pair_code) return set_err(ctx, MCGPU_ERR_INVALID, "null pair codes");
  auto I = std::make_unique<IntraHost>();
  I->n_bond = nb;
  I->n_angle = na;
  I->n_type = nt;
  I->max_intra_moves = t->max_intra_moves;
  I->max_bond_delta = t->max_bond_delta;
  I->max_angle_delta = t->max_angle_delta;
  I->step = t->step_num;
  I->bstart.assign(t->mol_bond_start, t->mol_bond_start + n_mol);
  I->bcount.assign(t->mol_bond_count, t->mol_bond_count + n_mol);
  I->astart.assign(t->mol_angle_start, t->mol_angle_start + n_mol);
  I->acount.assign(t->mol_angle_count, t->mol_angle_count + n_mol);
  I->bvar.assign(t->bond_var, t->bond_var + nb);
  I->avar.assign(t->angle_var, t->angle_var + na);
  for (int k = 0; k < nb; k++) I->flex_bonds |= t->bond_var[k] != 0;
  for (int k = 0; k < na; k++) I->flex_angles |= t->angle_var[k] != 0;
  // partitions, checked indexes
  std::vector<int> b_part(std::max(nb, 1), -1), a_part(std::max(na, 1), -1);
  std::vector<unsigned char> part;
  std::vector<int> p;
  for (int m = 0; m < n_mol; m++) {
    const int s = mol_start[m], len = mol_len[m];
    const int bs = I->bstart[m], bc = I->bcount[m], as = I->astart[m], ac = I->acount[m];
    if (bs < 0 || bc < 0 || bs + bc > nb || as < 0 || ac < 0 || as + ac > na)
      return set_err(ctx, MCGPU_ERR_INVALID, "molecule %d: bond or angle range outside the rows",
                     m);
    if (t->mol_type[m] < 0 || t->mol_type[m] >= nt)
      return set_err(ctx, MCGPU_ERR_INVALID, "molecule %d: type %d out of [0,%d)", m,
                     t->mol_type[m], nt);
    auto inside = [&](int a) { return a >= s && a < s + len; };
    for (int k = bs; k < bs + bc; k++)
      if (!inside(t->bond_a1[k]) || !inside(t->bond_a2[k]))
        return set_err(ctx, MCGPU_ERR_INVALID, "bond %d: atoms %d-%d outside molecule %d", k,
                       t->bond_a1[k], t->bond_a2[k], m);
    for (int k = as; k < as + ac; k++) {
      if (!inside(t->angle_a1[k]) || !inside(t->angle_a2[k]))
        return set_err(ctx, MCGPU_ERR_INVALID, "angle %d: ends %d, %d outside molecule %d", k,
                       t->angle_a1[k], t->angle_a2[k], m);
      if (t->angle_mid[k] < 0 || t->angle_mid[k] >= n_atom)
        return set_err(ctx, MCGPU_ERR_INVALID, "angle %d: middle atom %d out of [0,%d)", k,
                       t->angle_mid[k], n_atom);
    }
    for (int k = bs; k < bs + bc; k++) {
      p.resize(len);
      for (int i = 0; i < len; i++) p[i] = i;
      for (int o = bs; o < bs + bc; o++) {
        if (o == k) continue;
        int r1 = uf_find(p, t->bond_a1[o] - s), r2 = uf_find(p, t->bond_a2[o] - s);
        if (r1 != r2) p[r1] = r2;
      }
      const int side1 = uf_find(p, t->bond_a1[k] - s), side2 = uf_find(p, t->bond_a2[k] - s);
      if (side1 == side2) continue;
      b_part[k] = (int)part.size();
      for (int i = 0; i < len; i++) part.push_back(uf_find(p, i) == side2 ? 1 : 0);
    }
    for (int k = as; k < as + ac; k++) {
      const int mid = t->angle_mid[k];
      p.resize(len);
      for (int i = 0; i < len; i++) p[i] = i;
      for (int o = bs; o < bs + bc; o++) {
        if (t->bond_a1[o] == mid || t->bond_a2[o] == mid) continue;
        int r1 = uf_find(p, t->bond_a1[o] - s), r2 = uf_find(p, t->bond_a2[o] - s);
        if (r1 != r2) p[r1] = r2;
      }
      const int g1 = uf_find(p, t->angle_a1[k] - s), g2 = uf_find(p, t->angle_a2[k] - s);
      if (g1 == g2) continue;
      a_part[k] = (int)part.size();
      for (int i = 0; i < len; i++) {
        const int g = uf_find(p, i);
        part.push_back(g == g1 ? 1 : (g == g2 ? 2 : 0));
      }
    }
  }
  cudaError_t e = cudaSuccess;
  auto up = [&](auto* src, size_t n) {
    using T = std::remove_const_t<std::remove_pointer_t<decltype(src)>>;
    T* d = dalloc<T>(n, &e);
    I->allocs.push_back(d);
    if (e == cudaSuccess && n) e = cudaMemcpy(d, src, n * sizeof(T), cudaMemcpyHostToDevice);
    return d;
  };
  IntraRows& R = I->R;
  R.n_bond = nb;
  R.n_angle = na;
  R.flex_bonds = I->flex_bonds;
  R.flex_angles = I->flex_angles;
  R.b_a1 = up(t->bond_a1, nb);
  R.b_a2 = up(t->bond_a2, nb);
  R.b_var = up(t->bond_var, nb);
  R.b_part = up(b_part.data(), nb);
  R.b_k = up(t->bond_k, nb);
  R.b_eq = up(t->bond_eq, nb);
  R.b_len = up(t->bond_len, nb);
  R.b_len_rb = up(t->bond_len, nb);
  R.a_a1 = up(t->angle_a1, na);
  R.a_a2 = up(t->angle_a2, na);
  R.a_mid = up(t->angle_mid, na);
  R.a_var = up(t->angle_var, na);
  R.a_part = up(a_part.data(), na);
  R.a_k = up(t->angle_k, na);
  R.a_eq = up(t->angle_eq, na);
  R.a_size = up(t->angle_size, na);
  R.a_size_rb = up(t->angle_size, na);
  R.m_bstart = up(t->mol_bond_start, n_mol);
  R.m_bcount = up(t->mol_bond_count, n_mol);
  R.m_astart = up(t->mol_angle_start, n_mol);
  R.m_acount = up(t->mol_angle_count, n_mol);
  R.m_type = up(t->mol_type, n_mol);
  R.t_natom = up(t->type_natom, nt);
  R.t_off = up(t_off.data(), nt);
  R.code = up(t->pair_code, (size_t)codes);
  R.part = up(part.data(), part.size());
  I->dout = dalloc<double>(2, &e);
  I->allocs.push_back(I->dout);
  if (e == cudaSuccess) e = cudaMallocHost((void**)&I->hout, 2 * sizeof(double));
  if (e != cudaSuccess)
    return set_err(ctx, MCGPU_ERR_NOMEM, "topology upload failed: %s", cudaGetErrorString(e));
  *out = std::move(I);
  return MCGPU_OK;
}

cudaError_t launch_intra_energy(const Pool& P, const IntraRows& R, int chain, int mol,
                                double* out, cudaStream_t st) {
  k_intra_energy<<<1, kIntraThreads, 0, st>>>(P, R, chain, mol, out);
  return cudaGetLastError();
}

cudaError_t launch_intra_ops(const Pool& P, const IntraRows& R, int chain, const IntraOps& ops,
                             double* out, cudaStream_t st) {
  k_intra_ops<<<1, kIntraThreads, 0, st>>>(P, R, chain, ops, out);
  return cudaGetLastError();
}

cudaError_t launch_intra_rollback(const Pool& P, const IntraRows& R, int chain, int mol,
                                  cudaStream_t st) {
  k_intra_rollback<<<1, kIntraThreads, 0, st>>>(P, R, chain, mol);
  return cudaGetLastError();
}

cudaError_t launch_plain_steps(bool f64, const LoopTask* tasks, int n_tasks, int n_steps,
                               SmemShape sh, cudaStream_t st) {
  if (n_tasks <= 0) return cudaSuccess;
  const int bytes = sh.bytes();
  if (f64) {
    cudaFuncSetAttribute(k_plain_steps<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    k_plain_steps<true><<<n_tasks, kLoopThreads, bytes, st>>>(tasks, n_steps, sh);
  } else {
    cudaFuncSetAttribute(k_plain_steps<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    k_plain_steps<false><<<n_tasks, kLoopThreads, bytes, st>>>(tasks, n_steps, sh);
  }
  return cudaGetLastError();
}

cudaError_t launch_intra_add(const Pool& P, const IntraRows& R, int n_mol, double* emol,
                             cudaStream_t st) {
  if (n_mol <= 0) return cudaSuccess;
  k_intra_add<<<n_mol, kIntraThreads, 0, st>>>(P, R, emol);
  return cudaGetLastError();
}

}  // namespace mcgpu
