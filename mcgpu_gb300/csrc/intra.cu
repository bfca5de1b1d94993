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
// part), no cutoff, zero at r = 0.
__device__ __forceinline__ double intra_pair(const Pool& P, int i, int j, const ChainHdr& H) {
  const double dx = make_periodic(__dsub_rn(P.x[j], P.x[i]), H.L[0]);
  const double dy = make_periodic(__dsub_rn(P.y[j], P.y[i]), H.L[1]);
  const double dz = make_periodic(__dsub_rn(P.z[j], P.z[i]), H.L[2]);
  const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
  const double r = sqrt(r2);
  double lj = 0.0, c = 0.0;
  if (r2 != 0.0) {
    const double ss = P.sig[i] * P.sig[j], ee = P.eps[i] * P.eps[j];
    const double sigma = sqrt(ss >= 0 ? ss : -ss);
    const double eps = sqrt(ee >= 0 ? ee : -ee);
    const double s2 = sigma * sigma / r2;
    const double s6 = s2 * s2 * s2;
    lj = 4.0 * eps * (s6 * s6 - s6);
  }
  if (r != 0.0) c = (P.q[i] * P.q[j] * 332.06) / r;
  return lj + c;
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

__global__ void __launch_bounds__(kIntraThreads) k_intra_ops(Pool P, IntraRows R, int chain,
                                                             IntraOps ops, double* out) {
  __shared__ double red[3 * (kIntraThreads / 32)];
  __shared__ double sv[9];
  const ChainHdr& H = P.hdr[chain];
  const int mol = ops.mol, m = H.mol0 + mol;
  const int a0 = P.mstart[m], len = P.mlen[m] & 255;
  const int tid = threadIdx.x;
  if (ops.flags & kIntraSave) {
    // SimCalcs::saveBonds / saveAngles (SimulationStep.cpp:678-701)
    for (int k = R.m_bstart[mol] + tid; k < R.m_bstart[mol] + R.m_bcount[mol]; k += blockDim.x)
      R.b_len_rb[k] = R.b_len[k];
    for (int k = R.m_astart[mol] + tid; k < R.m_astart[mol] + R.m_acount[mol]; k += blockDim.x)
      R.a_size_rb[k] = R.a_size[k];
  }
  __syncthreads();
  if (ops.flags & kIntraEnergyBefore) {
    const double e = intra_energy(P, R, H, mol, red);
    if (tid == 0) out[0] = e;
  }
  bool moved = false;
  for (int k = 0; k < ops.n; k++) {
    const int i = ops.idx[k];
    if (ops.kind == 0) {
      // SimCalcs::stretchBond (SimulationStep.cpp:257-315)
      const int b = R.m_bstart[mol] + i;
      const int off = R.b_part[b];
      if (off < 0) continue;  // a ring: the reference returns before moving
      const double dist = ops.amt[k];
      if (tid == 0) {
        const int e1 = H.atom0 + R.b_a1[b], e2 = H.atom0 + R.b_a2[b];
        const double vx = __dsub_rn(P.x[e2], P.x[e1]);
        const double vy = __dsub_rn(P.y[e2], P.y[e1]);
        const double vz = __dsub_rn(P.z[e2], P.z[e1]);
        double d = __dadd_rn(0.0, __dmul_rn(vx, vx));
        d = __dadd_rn(d, __dmul_rn(vy, vy));
        d = __dadd_rn(d, __dmul_rn(vz, vz));
        d = __dsqrt_rn(d);
        sv[0] = __ddiv_rn(__ddiv_rn(vx, d), 2.0);
        sv[1] = __ddiv_rn(__ddiv_rn(vy, d), 2.0);
        sv[2] = __ddiv_rn(__ddiv_rn(vz, d), 2.0);
        R.b_len[b] = __dadd_rn(R.b_len[b], dist);
      }
      __syncthreads();
      if (tid < len) {
        const int a = a0 + tid;
        const double sx = __dmul_rn(sv[0], dist), sy = __dmul_rn(sv[1], dist),
                     sz = __dmul_rn(sv[2], dist);
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
      moved = true;
      __syncthreads();
    } else {
      // SimCalcs::expandAngle (SimulationStep.cpp:148-239)
      const int g = R.m_astart[mol] + i;
      const int off = R.a_part[g];
      if (off < 0) continue;  // both ends in one component
      if (tid == 0) {
        const int e1 = H.atom0 + R.a_a1[g], e2 = H.atom0 + R.a_a2[g],
                  md = H.atom0 + R.a_mid[g];
        const double m0 = P.x[md], m1 = P.y[md], m2 = P.z[md];
        const double p0 = __dsub_rn(m0, P.x[e1]), p1 = __dsub_rn(m1, P.y[e1]),
                     p2 = __dsub_rn(m2, P.z[e1]);
        const double q0 = __dsub_rn(m0, P.x[e2]), q1 = __dsub_rn(m1, P.y[e2]),
                     q2 = __dsub_rn(m2, P.z[e2]);
        double n0 = __dsub_rn(__dmul_rn(p1, q2), __dmul_rn(q1, p2));
        double n1 = __dsub_rn(__dmul_rn(q0, p2), __dmul_rn(p0, q2));
        double n2 = __dsub_rn(__dmul_rn(p0, q1), __dmul_rn(q0, p1));
        double nl = __dadd_rn(0.0, __dmul_rn(n0, n0));
        nl = __dadd_rn(nl, __dmul_rn(n1, n1));
        nl = __dadd_rn(nl, __dmul_rn(n2, n2));
        nl = __dsqrt_rn(nl);
        sv[0] = __ddiv_rn(n0, nl);
        sv[1] = __ddiv_rn(n1, nl);
        sv[2] = __ddiv_rn(n2, nl);
        sv[3] = m0;
        sv[4] = m1;
        sv[5] = m2;
        R.a_size[g] = __dadd_rn(R.a_size[g], ops.amt[k]);
      }
      __syncthreads();
      if (tid < len) {
        const int lab = R.part[off + tid];
        if (lab) {
          const double cs = lab == 1 ? ops.c1[k] : ops.c2[k];
          const double sn = lab == 1 ? ops.s1[k] : ops.s2[k];
          const double omc = __dsub_rn(1.0, cs);
          const int a = a0 + tid;
          const double t0 = __dsub_rn(P.x[a], sv[3]), t1 = __dsub_rn(P.y[a], sv[4]),
                       t2 = __dsub_rn(P.z[a], sv[5]);
          double dot = __dadd_rn(0.0, __dmul_rn(t0, sv[0]));
          dot = __dadd_rn(dot, __dmul_rn(t1, sv[1]));
          dot = __dadd_rn(dot, __dmul_rn(t2, sv[2]));
          const double c0 = __dsub_rn(__dmul_rn(sv[1], t2), __dmul_rn(t1, sv[2]));
          const double c1 = __dsub_rn(__dmul_rn(t0, sv[2]), __dmul_rn(sv[0], t2));
          const double c2 = __dsub_rn(__dmul_rn(sv[0], t1), __dmul_rn(t0, sv[1]));
          const double u0 = __dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(sv[0], dot), omc),
                                                __dmul_rn(t0, cs)), __dmul_rn(c0, sn));
          const double u1 = __dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(sv[1], dot), omc),
                                                __dmul_rn(t1, cs)), __dmul_rn(c1, sn));
          const double u2 = __dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(sv[2], dot), omc),
                                                __dmul_rn(t2, cs)), __dmul_rn(c2, sn));
          P.x[a] = __dadd_rn(u0, sv[3]);
          P.y[a] = __dadd_rn(u1, sv[4]);
          P.z[a] = __dadd_rn(u2, sv[5]);
        }
      }
      moved = true;
      __syncthreads();
    }
  }
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
  const ChainHdr& H = P.hdr[chain];
  const int m = H.mol0 + mol;
  const int a0 = P.mstart[m], len = P.mlen[m] & 255;
  const double* rb = P.rb + (size_t)chain * 3 * H.max_len;
  for (int i = threadIdx.x; i < len; i += blockDim.x) {
    P.x[a0 + i] = rb[i];
    P.y[a0 + i] = rb[H.max_len + i];
    P.z[a0 + i] = rb[2 * H.max_len + i];
  }
  // SimCalcs::rollbackAngles / rollbackBonds (SimulationStep.cpp:751-775)
  for (int k = R.m_astart[mol] + threadIdx.x; k < R.m_astart[mol] + R.m_acount[mol];
       k += blockDim.x)
    R.a_size[k] = R.a_size_rb[k];
  for (int k = R.m_bstart[mol] + threadIdx.x; k < R.m_bstart[mol] + R.m_bcount[mol];
       k += blockDim.x)
    R.b_len[k] = R.b_len_rb[k];
  __syncthreads();
  refresh_flexible(P, H, m, red);
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

cudaError_t launch_intra_add(const Pool& P, const IntraRows& R, int n_mol, double* emol,
                             cudaStream_t st) {
  if (n_mol <= 0) return cudaSuccess;
  k_intra_add<<<n_mol, kIntraThreads, 0, st>>>(P, R, emol);
  return cudaGetLastError();
}

}  // namespace mcgpu
