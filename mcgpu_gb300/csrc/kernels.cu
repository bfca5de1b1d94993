// kernels.cu -- __global__ kernels of the trial-move energy path.
//
//   k_refresh_mirrors      FP32 mirrors from the FP64 master rows (upload)
//   k_mol_energy<F64>      calcMolecularEnergyContribution over a candidate
//                          range, many CTAs, deterministic last-CTA sum
//   k_move_energies<F64>   old energy + move + new energy in one launch
//   k_change_molecule      the move alone (saves the rollback copy)
//   k_rollback             restores the rollback copy
//   k_mol_pair_sums<F64>   E(m, j>m) per molecule of every chain
//   k_chain_sums           per-chain ordered sum of the above
//   k_chain_steps          persistent Metropolis steps of many chains:
//                          Philox proposal, staging, screen, pairs, FP64
//                          dE, decision and commit without leaving the GPU
#include "kernels.cuh"

namespace mcgpu {

// ---- mirrors ---------------------------------------------------------------

__global__ void k_refresh_mirrors(Pool P, const int* mol_chain, int n_mol_total) {
  const int m = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (m >= n_mol_total) return;
  refresh_molecule(P, P.hdr[mol_chain[m]], m, threadIdx.x & 31, 32);
}

// ---- deterministic last-CTA sum ------------------------------------------

// Thread 0 of a CTA: publishes its writes and reports whether this CTA is
// the last of the grid to arrive (it then owns the ordered final sum).
__device__ bool arrive_last(unsigned* counter) {
  __threadfence();
  unsigned t = atomicAdd(counter, 1u);
  return t == gridDim.x - 1;
}

// ---- plain contract ---------------------------------------------------------

// Energy of molecule `curr` against chain-local candidates [start, n_mol)
// (BruteForceCalcs::calcMolecularEnergyContribution, BruteForceStep.cpp:
// 15-46).  Each CTA takes an equal slice of the candidates.
template <bool F64>
__global__ void __launch_bounds__(256) k_mol_energy(Pool P, int chain, int curr, int start,
                                                    SmemShape shape, double* partials,
                                                    unsigned* counter, double* out) {
  extern __shared__ __align__(16) char smem[];
  const ChainHdr& H = P.hdr[chain];
  Group g{(int)threadIdx.x, (int)blockDim.x, 1};
  GroupSmem s = shape.carve(smem);
  const int lane = threadIdx.x & 31, w = g.warp(), nw = g.nwarps();
  const int m = H.mol0 + curr;
  if (w == 0) stage(P, H, m, nullptr, s, lane);
  g.sync();
  const MovedInfo mi = load_moved(s);
  const int n_cand = H.n_mol - start;
  const int chunk = ((n_cand + gridDim.x - 1) / gridDim.x + 31) & ~31;
  const int cb = H.mol0 + start + blockIdx.x * chunk;
  const int ce = min(cb + chunk, H.mol0 + H.n_mol);
  double eo = 0.0, en = 0.0, ab = 0.0;
  long long np = 0;
  if (cb < ce) warp_eval<F64>(P, H, s, mi, cb, ce, w, nw, lane, H.tpm, eo, en, ab, np);
  group_reduce(g, s, eo, en, ab, np);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = eo;
    if (arrive_last(counter)) {
      __threadfence();
      double sum = 0.0;
      for (unsigned b = 0; b < gridDim.x; b++) sum += ((volatile double*)partials)[b];
      out[0] = sum;
      *counter = 0;
    }
  }
}

// Old energy, the move, and new energy of molecule `mol` in one launch
// (Simulation.cpp:244-250).  Every CTA stages the same proposed placement;
// the CTA that finishes last saves the rollback copy and commits.
template <bool F64>
__global__ void __launch_bounds__(256) k_move_energies(Pool P, int chain, int mol, Proposal prop,
                                                       SmemShape shape, double* partials,
                                                       unsigned* counter, double* out) {
  extern __shared__ __align__(16) char smem[];
  const ChainHdr& H = P.hdr[chain];
  Group g{(int)threadIdx.x, (int)blockDim.x, 1};
  GroupSmem s = shape.carve(smem);
  const int lane = threadIdx.x & 31, w = g.warp(), nw = g.nwarps();
  const int m = H.mol0 + mol;
  if (w == 0) stage(P, H, m, &prop, s, lane);
  g.sync();
  const MovedInfo mi = load_moved(s);
  const int chunk = ((H.n_mol + gridDim.x - 1) / gridDim.x + 31) & ~31;
  const int cb = H.mol0 + blockIdx.x * chunk;
  const int ce = min(cb + chunk, H.mol0 + H.n_mol);
  double eo = 0.0, en = 0.0, ab = 0.0;
  long long np = 0;
  if (cb < ce) warp_eval<F64>(P, H, s, mi, cb, ce, w, nw, lane, H.tpm, eo, en, ab, np);
  group_reduce(g, s, eo, en, ab, np);
  __shared__ int last;
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = eo;
    partials[2 * blockIdx.x + 1] = en;
    last = arrive_last(counter) ? 1 : 0;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  if (w == 0) {
    double* rb = P.rb + (size_t)chain * 3 * H.max_len;
    for (int i = lane; i < mi.len; i += 32) {
      rb[i] = s.ox[i];
      rb[H.max_len + i] = s.oy[i];
      rb[2 * H.max_len + i] = s.oz[i];
    }
    commit(P, s, mi, lane);
    if (lane == 0) {
      double so = 0.0, sn = 0.0;
      for (unsigned b = 0; b < gridDim.x; b++) {
        so += ((volatile double*)partials)[2 * b];
        sn += ((volatile double*)partials)[2 * b + 1];
      }
      out[0] = so;
      out[1] = sn;
      *counter = 0;
    }
  }
}

// The move alone (SimCalcs::intermolecularMove with supplied draws).
__global__ void k_change_molecule(Pool P, int chain, int mol, Proposal prop, SmemShape shape) {
  extern __shared__ __align__(16) char smem[];
  const ChainHdr& H = P.hdr[chain];
  GroupSmem s = shape.carve(smem);
  const int lane = threadIdx.x & 31;
  stage(P, H, H.mol0 + mol, &prop, s, lane);
  __syncwarp();
  const MovedInfo mi = load_moved(s);
  double* rb = P.rb + (size_t)chain * 3 * H.max_len;
  for (int i = lane; i < mi.len; i += 32) {
    rb[i] = s.ox[i];
    rb[H.max_len + i] = s.oy[i];
    rb[2 * H.max_len + i] = s.oz[i];
  }
  commit(P, s, mi, lane);
}

// SimCalcs::rollback (SimulationStep.cpp:731-749) plus the mirrors.
__global__ void k_rollback(Pool P, int chain, int mol) {
  const ChainHdr& H = P.hdr[chain];
  const int m = H.mol0 + mol;
  const int a0 = P.mstart[m], len = P.mlen[m] & 255;
  const double* rb = P.rb + (size_t)chain * 3 * H.max_len;
  const int lane = threadIdx.x & 31;
  for (int i = lane; i < len; i += 32) {
    P.x[a0 + i] = rb[i];
    P.y[a0 + i] = rb[H.max_len + i];
    P.z[a0 + i] = rb[2 * H.max_len + i];
  }
  __syncwarp();
  refresh_molecule(P, H, m, lane, 32);
}

// E(m, j > m) for pool molecule m = blockIdx.x + m_begin: one term of
// SimulationStep::calcSystemEnergy (SimulationStep.cpp:47-48).
template <bool F64>
__global__ void __launch_bounds__(256) k_mol_pair_sums(Pool P, const int* mol_chain, int m_begin,
                                                       SmemShape shape, double* emol,
                                                       long long* pairs) {
  extern __shared__ __align__(16) char smem[];
  const int m = m_begin + blockIdx.x;
  const ChainHdr& H = P.hdr[mol_chain[m]];
  Group g{(int)threadIdx.x, (int)blockDim.x, 1};
  GroupSmem s = shape.carve(smem);
  const int lane = threadIdx.x & 31, w = g.warp(), nw = g.nwarps();
  if (w == 0) stage(P, H, m, nullptr, s, lane);
  g.sync();
  const MovedInfo mi = load_moved(s);
  double eo = 0.0, en = 0.0, ab = 0.0;
  long long np = 0;
  warp_eval<F64>(P, H, s, mi, m + 1, H.mol0 + H.n_mol, w, nw, lane, H.tpm, eo, en, ab, np);
  group_reduce(g, s, eo, en, ab, np);
  if (threadIdx.x == 0) {
    emol[m] = eo;
    if (pairs) pairs[m] = np;
  }
}

// Ordered per-chain sum of emol: thread t adds every blockDim-th term from
// t, then a fixed tree; one CTA per chain.
__global__ void k_chain_sums(Pool P, const double* emol, double* out) {
  __shared__ double red[256];
  const ChainHdr& H = P.hdr[blockIdx.x];
  double acc = 0.0;
  for (int i = threadIdx.x; i < H.n_mol; i += blockDim.x) acc += emol[H.mol0 + i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int off = blockDim.x >> 1; off > 0; off >>= 1) {
    if ((int)threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

// Sets every chain's running energy from out[] (the start of a run).
__global__ void k_set_energy(Pool P, const double* e) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < P.n_chains) P.hdr[c].energy = e[c];
}

// ---- device-resident Metropolis -------------------------------------------

// Persistent kernel: groups of `gwarps` warps pull chain tasks from `queue`
// (task k runs chain order[k]) and advance each by n_steps steps.  A step:
// warp 0 draws the Philox proposal and stages the molecule (one group
// barrier), every warp screens and evaluates its share of candidates into
// FP64 sums, a group reduction (one barrier) gives E_old, E_new; warp 0
// decides (dE < 0, else exp(-dE/kT) >= u, SimulationStep.cpp:794-803) and
// commits.  If trace != nullptr, step st of chain c is recorded at
// trace[c * trace_stride + trace_off + st].
__global__ void __launch_bounds__(512) k_chain_steps(Pool P, int n_steps, unsigned* queue,
                                                     const int* order, int n_tasks, int gwarps,
                                                     SmemShape shape, mcgpu_trace* trace,
                                                     int trace_off, int trace_stride) {
  extern __shared__ __align__(16) char smem[];
  const int gsize = gwarps * 32;
  const int gid = threadIdx.x / gsize;
  Group g{(int)threadIdx.x - gid * gsize, gsize, 1 + gid};
  GroupSmem s = shape.carve(smem + gid * shape.bytes());
  const int lane = threadIdx.x & 31, w = g.warp(), nw = g.nwarps();
  for (;;) {
    if (g.tid == 0) s.misc[31] = (int)atomicAdd(queue, 1u);
    g.sync();
    const int task = s.misc[31];
    if (task >= n_tasks) break;
    const int c = order[task];
    ChainHdr* Hp = P.hdr + c;
    const ChainHdr& H = *Hp;
    double energy = H.energy;
    long long acc = 0, npairs = 0;
    int ties = 0;
    const unsigned long long step0 = H.step;
    for (int st = 0; st < n_steps; st++) {
      Proposal p;
      if (w == 0) {
        if (lane == 0)
          p = draw_proposal(H.seed, H.chain_id, step0 + st, H.n_mol, P.mlen + H.mol0, H.max_t,
                            H.max_r, H.rot_mode);
        p.mol = __shfl_sync(~0u, p.mol, 0);
        p.vertex = __shfl_sync(~0u, p.vertex, 0);
        p.mode = H.rot_mode;
        p.dx = __shfl_sync(~0u, p.dx, 0);
        p.dy = __shfl_sync(~0u, p.dy, 0);
        p.dz = __shfl_sync(~0u, p.dz, 0);
        p.r0 = __shfl_sync(~0u, p.r0, 0);
        p.r1 = __shfl_sync(~0u, p.r1, 0);
        p.r2 = __shfl_sync(~0u, p.r2, 0);
        p.r3 = __shfl_sync(~0u, p.r3, 0);
        stage(P, H, H.mol0 + p.mol, &p, s, lane);
        if (lane == 0) s.miscd[2] = p.u;
      }
      g.sync();
      const MovedInfo mi = load_moved(s);
      double eo = 0.0, en = 0.0, ab = 0.0;
      long long np = 0;
      warp_eval<false>(P, H, s, mi, H.mol0, H.mol0 + H.n_mol, w, nw, lane, H.tpm, eo, en, ab, np);
      group_reduce(g, s, eo, en, ab, np);
      // Decision guard band: when exp(-dE/kT) lies within the FP32 rounding
      // bound of u, the group re-evaluates both placements with FP64 pairs
      // (the reference's arithmetic) and decides on that dE, so decisions
      // match the FP64 path outside |-dE/kT - ln u| < ~1e-12.
      int tie = 0;
      {
        const float u = (float)s.miscd[2];
        const double bound = kTieRel * ab + 1e-9;
        const double de32 = en - eo;
        if (de32 >= -bound) {
          const float pf = expf(-(float)(fmax(de32, 0.0) / H.kT));
          tie = fabsf(pf - u) <= pf * (float)(1.5 * bound / H.kT) + 4e-6f;
        }
      }
      if (tie) {
        g.sync();
        eo = 0.0;
        en = 0.0;
        double ab2 = 0.0;
        long long np2 = 0;
        warp_eval<true>(P, H, s, mi, H.mol0, H.mol0 + H.n_mol, w, nw, lane, H.tpm, eo, en, ab2,
                        np2);
        group_reduce(g, s, eo, en, ab2, np2);
      }
      if (w == 0) {
        const double de = en - eo;
        int ok = 0;
        if (lane == 0) ok = (de < 0) || (exp(-(de) / H.kT) >= p.u);
        ok = __shfl_sync(~0u, ok, 0);
        if (ok) commit(P, s, mi, lane);
        if (lane == 0) {
          if (ok) {
            energy += de;
            acc++;
          }
          npairs += np;
          ties += tie;
          if (trace) {
            mcgpu_trace t;
            t.mol = mi.mol - H.mol0;
            t.accepted = ok;
            t.e_old = eo;
            t.e_new = en;
            t.de = de;
            t.u = p.u;
            t.fp64 = tie;
            t.pad0 = 0;
            trace[(size_t)c * trace_stride + trace_off + st] = t;
          }
        }
        __syncwarp();
      }
    }
    if (g.tid == 0) {
      Hp->energy = energy;
      Hp->step = step0 + n_steps;
      Hp->accepted += acc;
      Hp->pairs += npairs;
      Hp->ties += ties;
    }
    g.sync();
  }
}

// ---- host launchers (template kernels are instantiated here) --------------

cudaError_t launch_mol_energy(bool f64, int grid, int threads, SmemShape sh, cudaStream_t st,
                              Pool P, int chain, int curr, int start, double* partials,
                              unsigned* counter, double* out) {
  if (f64)
    k_mol_energy<true><<<grid, threads, sh.bytes(), st>>>(P, chain, curr, start, sh, partials,
                                                          counter, out);
  else
    k_mol_energy<false><<<grid, threads, sh.bytes(), st>>>(P, chain, curr, start, sh, partials,
                                                           counter, out);
  return cudaGetLastError();
}

cudaError_t launch_move_energies(bool f64, int grid, int threads, SmemShape sh, cudaStream_t st,
                                 Pool P, int chain, int mol, Proposal prop, double* partials,
                                 unsigned* counter, double* out) {
  if (f64)
    k_move_energies<true><<<grid, threads, sh.bytes(), st>>>(P, chain, mol, prop, sh, partials,
                                                             counter, out);
  else
    k_move_energies<false><<<grid, threads, sh.bytes(), st>>>(P, chain, mol, prop, sh, partials,
                                                              counter, out);
  return cudaGetLastError();
}

cudaError_t launch_mol_pair_sums(bool f64, int grid, int threads, SmemShape sh, cudaStream_t st,
                                 Pool P, const int* mol_chain, int m_begin, double* emol,
                                 long long* pairs) {
  if (f64)
    k_mol_pair_sums<true><<<grid, threads, sh.bytes(), st>>>(P, mol_chain, m_begin, sh, emol, pairs);
  else
    k_mol_pair_sums<false><<<grid, threads, sh.bytes(), st>>>(P, mol_chain, m_begin, sh, emol,
                                                              pairs);
  return cudaGetLastError();
}

}  // namespace mcgpu
