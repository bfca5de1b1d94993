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
#include "chain.cuh"

namespace mcgpu {

// ---- mirrors ---------------------------------------------------------------

__global__ void k_refresh_mirrors(Pool P, const int* mol_chain, int m_begin, int m_end) {
  const int m = m_begin + blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (m >= m_end) return;
  refresh_molecule(P, P.hdr[mol_chain[m]], m, threadIdx.x & 31, 32);
}

// The FP64 pair terms' per-atom blending factors (blend64).
__global__ void k_blend_rows(Pool P, int n_atom) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a < n_atom) P.blend[a] = blend64(P.sig[a], P.eps[a]);
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
                                                    unsigned* counter, double* out,
                                                    long long* pairs) {
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
    if (pairs) atomicAdd((unsigned long long*)pairs, (unsigned long long)np);
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
                                                       unsigned* counter, double* out,
                                                       long long* pairs) {
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
    if (pairs) atomicAdd((unsigned long long*)pairs, (unsigned long long)np);
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

// Running energy of chain c from its emol terms: the ordered sum of
// k_chain_sums for one chain (a served job entering the pool).
__global__ void k_chain_energy1(Pool P, int c, const double* emol) {
  __shared__ double red[256];
  ChainHdr& H = P.hdr[c];
  double acc = 0.0;
  for (int i = threadIdx.x; i < H.n_mol; i += blockDim.x) acc += emol[H.mol0 + i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int off = blockDim.x >> 1; off > 0; off >>= 1) {
    if ((int)threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0) H.energy = red[0];
}

// ---- device-resident Metropolis -------------------------------------------

// Puts every molecule of the pool in the device-resident chain state:
// anchor = its first primary atom in fixed point, offsets = FP32 (atom -
// anchor), template = offsets, quaternion = identity; then snaps the FP64
// rows to that state (x = anchor + offset, each moved by < 1e-7 A) so both
// descriptions agree exactly.  One warp per molecule.
__global__ void k_chain_init(Pool P, const int* mol_chain, int m_begin, int m_end) {
  const int m = m_begin + blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (m >= m_end) return;
  const ChainHdr& H = P.hdr[mol_chain[m]];
  const int lane = threadIdx.x & 31;
  const int a0 = P.mstart[m], len = P.mlen[m] & 255;
  const int2 pi = P.mpi[m];
  const int an = P.pidx[pi.x];
  const double ax = P.x[an], ay = P.y[an], az = P.z[an];
  const uint4 A = fixpos(ax, ay, az, H);
  __syncwarp();
  for (int i = lane; i < len; i += 32) {
    const int a = a0 + i;
    const float w = P.aoff[a].w;
    const float4 o = make_float4((float)(P.x[a] - ax), (float)(P.y[a] - ay), (float)(P.z[a] - az), w);
    P.aoff[a] = o;
    P.aofl[a] = make_float4(0.f, 0.f, 0.f, 0.f);
    P.atpl[a] = make_float4(o.x, o.y, o.z, 0.f);
  }
  __syncwarp();
  for (int i = lane; i < len; i += 32) {
    const int a = a0 + i;
    const double3 x = chain_pos3(A, P.aoff[a], H);
    P.x[a] = x.x;
    P.y[a] = x.y;
    P.z[a] = x.z;
  }
  __syncwarp();
  for (int k = lane; k < pi.y; k += 32) {
    const int q = P.pidx[pi.x + k];
    P.ppos[pi.x + k] = wrap_pos(P.x[q], P.y[q], P.z[q], H);
  }
  if (lane == 0) {
    P.mfix[m] = A;
    P.mq[m] = make_float4(1.f, 0.f, 0.f, 0.f);
  }
}

// FP64 rows of every atom from the chain state (for downloads, FP64
// recomputes and the plain entry points).  One thread per atom.
__global__ void k_chain_export(Pool P, const int* mol_chain, const int* atom_mol, int a_begin,
                               int a_end) {
  const int a = a_begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= a_end) return;
  const int m = atom_mol[a];
  const ChainHdr& H = P.hdr[mol_chain[m]];
  const double3 x = chain_pos3(P.mfix[m], P.aoff[a], H);
  P.x[a] = x.x;
  P.y[a] = x.y;
  P.z[a] = x.z;
}

// Persistent kernel: groups of `gwarps` warps pull chain tasks from `queue`
// (task k runs chain order[k]) and advance each by n_steps steps on the
// chain state.  A step: every warp screens its share of the candidates
// against the move staged in FP32 during the previous step and evaluates
// the in-range ones (FP32 pair terms, double-float sums); the last warp then
// stages the next move into the next of three shared-memory slots; one
// group reduction (the step's barrier) gives every thread E_old, E_new.
// Outside a guard band around the acceptance threshold the decision
// (dE < 0, else exp(-dE/kT) >= u, SimulationStep.cpp:794-803) is taken in
// FP32; inside it the group re-evaluates both placements with FP64 pairs and
// decides on that.  Every warp takes the decision and writes the accepted
// placement itself and goes on to the next step; warp 0 keeps the running
// energy and the counters.  With cache_n > 0 each group keeps its chain's
// primary screen positions in shared memory.  If trace != nullptr, step st
// of chain c is recorded at trace[c * trace_stride + trace_off + st].  The
// staging warp draws the moves of 32 steps at once (one per lane) into
// shared memory; when a commit moves the molecule of the move staged next,
// warp 0 stages it again (one more barrier).  lanes_cap > 0 caps the lanes
// per neighbour molecule of every chain.
__device__ __forceinline__ void chain_steps(Pool P, int n_steps, unsigned* queue,
                                            const int* order, int n_tasks, int gwarps,
                                            SmemShape shape, mcgpu_trace* trace, int trace_off,
                                            int trace_stride, int lanes_cap, char* smem) {
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
    float4* pcache = (s.pc && H.simple_prim && H.n_mol <= shape.cache_n) ? s.pc : nullptr;
    if (pcache)
      for (int i = g.tid; i < H.n_mol; i += gsize) pcache[i] = P.ppos[H.pidx0 + i];
    if (H.uniform)
      for (int i = g.tid; i < H.ulen; i += gsize) s.teq[i] = P.aeq[H.atom0 + i];
    g.sync();
    // the chain's LJ mask, read by the pair batches after the next barrier
    // (kept in the header rather than in a register across the step loop)
    if (g.tid == 0) Hp->ljmask = uniform_lj_mask(P, H, s.teq);
    int full_scans = 0;
    // the accepted dE of this task and their FP32 error bounds, each summed
    // in double-float (FP64 costs 64 FP32 issue slots on GB300); both join
    // the FP64 header values once, at the task's end
    float de_h = 0.f, de_l = 0.f, err_h = 0.f, err_l = 0.f;
    long long acc_n = 0, npairs = 0;
    int ties = 0;
    const unsigned long long step0 = H.step;
    // the Verlet list stays valid while no accepted molecule has moved beyond
    // skin/2 of the build (every thread keeps the same flag)
    bool nl_ok = H.nl_on && H.nl_valid;
    // lanes per neighbour molecule: the cap, else one lane for a chain of
    // one species of at most 4 atoms (the single-lane pair batch), else the
    // power of two at or above its largest molecule
    const int T = lanes_cap > 0 ? min(lanes_cap, H.tpm)
                                : ((H.uniform && H.ulen <= 4 && !H.precise) ? 1 : H.tpm);
    MoveF* props = (MoveF*)s.props;
    int my_steps = n_steps;
    if (H.step_limit > 0)
      my_steps = (int)max(0LL, min((long long)n_steps, H.step_limit - (long long)step0));
    // step st's move is staged in slot st % 3 (the last warp stages step
    // st + 1 during step st; slot (st + 2) % 3 = (st - 1) % 3 is rewritten
    // only after every warp has passed step st's reduction barrier, so no
    // warp still commits from it)
    const int sb = shape.ahead_bytes();
    auto slot = [&](int k) { return shape.ahead_slot(s.ahead + k * sb); };
    // moves are drawn 32 steps at a time (one per lane) by the staging warp
    auto draw32 = [&](int st0) {
      if (st0 + lane < my_steps)
        props[lane] = draw_move_f32(H.seed, H.chain_id, step0 + st0 + lane, H.n_mol,
                                    P.mlen + H.mol0, (float)H.max_t, (float)H.max_r, H.rot_mode);
      __syncwarp();
    };
    if (w == 0 && my_steps > 0) {
      draw32(0);
      stage_chain(P, H, props[0], slot(0), pcache, lane);
    }
    g.sync();
    for (int st = 0; st < my_steps; st++) {
      const int k = st % 3, kn = k == 2 ? 0 : k + 1;
      const GroupSmem ss = with_slot(s, slot(k));
      const MovedInfo mi = load_moved(ss);
      const float u = __int_as_float(ss.misc[kMiscU]);
      // Verlet list while it is valid and the trial placement stays within
      // skin/2 of the build; the full scan otherwise (same in-range set)
      const int trial_near = ss.misc[kMiscNlTrial];
      const bool use_list = nl_ok && trial_near;
      AccFF acc = {0.f, 0.f, 0.f, 0.f, 0.f, 0};
      // FP64-pair chains skip the FP32 evaluation: every step is taken by
      // the FP64 path below
      const bool f64all = H.fp64_pairs != 0;
      if (f64all) {
      } else if (use_list)
        warp_eval_chain(P, H, ss, mi, pcache, 0, P.nl_cnt[mi.mol], w, nw, lane, T, acc,
                        P.nl + (size_t)mi.mol * P.nl_stride);
      else
        warp_eval_chain(P, H, ss, mi, pcache, H.mol0, H.mol0 + H.n_mol, w, nw, lane, T, acc);
      // the last warp (with the fewest screen blocks) stages the next move
      // while the others finish their share
      if (w == nw - 1 && st + 1 < my_steps) {
        if (((st + 1) & 31) == 0) draw32(st + 1);
        stage_chain(P, H, props[(st + 1) & 31], slot(kn), pcache, lane);
      }
      // the step's one barrier; every thread ends with the same totals
      group_reduce_ff(g, ss, acc, st & 1);
      // FP32 decision unless the FP32 dE is within its rounding bound of the
      // threshold; the bound covers the pair terms' rounding (kTieRel of the
      // sum of magnitudes) and the FP32 difference of the two totals.
      const float de_f = __fadd_rn(__fsub_rn(acc.nh, acc.oh), __fsub_rn(acc.nl, acc.ol));
      const float bound = (float)kTieRel * acc.ab + 2.4e-7f * (fabsf(acc.nh) + fabsf(acc.oh)) + 1e-9f;
      const float pf = expf(-fmaxf(de_f, 0.f) * H.kTinvf);
      const int tie = f64all ||
                      ((de_f >= -bound) && (fabsf(pf - u) <= pf * (1.5f * bound * H.kTinvf) + 1e-6f));
      double e_old = 0.0, e_new = 0.0;
      int ok;
      if (tie) {
        if (w == 0) stage_chain_f64(P, H, ss, mi, lane);
        g.sync();
        double eo = 0.0, en = 0.0, ab2 = 0.0;
        long long np2 = 0;
        if (use_list)
          warp_eval_chain64(P, H, ss, mi, pcache, 0, P.nl_cnt[mi.mol], w, nw, lane, T, eo, en,
                            P.nl + (size_t)mi.mol * P.nl_stride);
        else
          warp_eval_chain64(P, H, ss, mi, pcache, H.mol0, H.mol0 + H.n_mol, w, nw, lane, T, eo,
                            en);
        group_reduce(g, ss, eo, en, ab2, np2, st & 1);
        e_old = eo;
        e_new = en;
        const double d64 = e_new - e_old;
        ok = (d64 < 0) || (exp(-d64 / H.kT) >= (double)u);
      } else {
        ok = (de_f < 0.f) || (pf >= u);
      }
      // every warp takes the same decision and writes the same new placement,
      // so each sees it in its next screen without waiting for the others
      if (ok) commit_chain(P, H, ss, mi, pcache, lane);
      __syncwarp();
      if (ok && !trial_near) nl_ok = false;
      if (w == 0 && lane == 0) {
        if (ok) {
          if (tie) {
            const double d64 = e_new - e_old;
            const float dh = (float)d64;
            ff_add2(de_h, de_l, dh, (float)(d64 - (double)dh));
            ff_add(err_h, err_l, 1e-12f * acc.ab);
          } else {
            ff_add2(de_h, de_l, acc.nh, acc.nl);
            ff_add2(de_h, de_l, -acc.oh, -acc.ol);
            ff_add(err_h, err_l, bound);
          }
          acc_n++;
        }
        if (H.nl_on && !use_list) full_scans++;
        npairs += acc.np;
        ties += tie;
        if (trace) {
          if (!tie) {
            e_old = (double)acc.oh + (double)acc.ol;
            e_new = (double)acc.nh + (double)acc.nl;
          }
          const double de = e_new - e_old;
          mcgpu_trace t;
          t.mol = mi.mol - H.mol0;
          t.accepted = ok;
          t.e_old = e_old;
          t.e_new = e_new;
          t.de = de;
          t.u = (double)u;
          t.fp64 = tie;
          t.pad0 = 0;
          trace[(size_t)c * trace_stride + trace_off + st] = t;
        }
      }
      // the next move was staged from rows this commit changes only if it
      // moves the same molecule (read from its slot: the staging warp may
      // already be drawing over props): warp 0 stages it again, all warps
      // wait (the condition is the same in every thread)
      if (st + 1 < my_steps && ok && slot(kn).misc[0] == mi.mol) {
        if (w == 0) stage_chain(P, H, props[(st + 1) & 31], slot(kn), pcache, lane);
        g.sync();
      }
    }
    if (g.tid == 0) {
      Hp->energy = H.energy + ((double)de_h + (double)de_l);
      Hp->run_err += (double)err_h + (double)err_l;
      Hp->step = step0 + my_steps;
      Hp->accepted += acc_n;
      Hp->pairs += npairs;
      Hp->ties += ties;
      if (H.nl_on) {
        Hp->nl_valid = nl_ok ? 1 : 0;
        Hp->nl_full += full_scans;
      }
    }
    g.sync();
  }
}

__global__ void __launch_bounds__(256, 2) k_chain_steps(Pool P, int n_steps, unsigned* queue,
                                                     const int* order, int n_tasks, int gwarps,
                                                     SmemShape shape, mcgpu_trace* trace,
                                                     int trace_off, int trace_stride,
                                                     int lanes_cap) {
  extern __shared__ __align__(16) char smem[];
  chain_steps(P, n_steps, queue, order, n_tasks, gwarps, shape, trace, trace_off, trace_stride,
              lanes_cap, smem);
}

// The same for one group of up to 16 warps per CTA (a single large chain:
// more warps per step, one CTA per SM).
__global__ void __launch_bounds__(512, 1) k_chain_steps_wide(Pool P, int n_steps,
                                                          unsigned* queue, const int* order,
                                                          int n_tasks, int gwarps,
                                                          SmemShape shape, mcgpu_trace* trace,
                                                          int trace_off, int trace_stride,
                                                          int lanes_cap) {
  extern __shared__ __align__(16) char smem[];
  chain_steps(P, n_steps, queue, order, n_tasks, gwarps, shape, trace, trace_off, trace_stride,
              lanes_cap, smem);
}

// ---- host launchers (template kernels are instantiated here) --------------

cudaError_t launch_mol_energy(bool f64, int grid, int threads, SmemShape sh, cudaStream_t st,
                              Pool P, int chain, int curr, int start, double* partials,
                              unsigned* counter, double* out, long long* pairs) {
  if (f64)
    k_mol_energy<true><<<grid, threads, sh.bytes(), st>>>(P, chain, curr, start, sh, partials,
                                                          counter, out, pairs);
  else
    k_mol_energy<false><<<grid, threads, sh.bytes(), st>>>(P, chain, curr, start, sh, partials,
                                                           counter, out, pairs);
  return cudaGetLastError();
}

cudaError_t launch_move_energies(bool f64, int grid, int threads, SmemShape sh, cudaStream_t st,
                                 Pool P, int chain, int mol, Proposal prop, double* partials,
                                 unsigned* counter, double* out, long long* pairs) {
  if (f64)
    k_move_energies<true><<<grid, threads, sh.bytes(), st>>>(P, chain, mol, prop, sh, partials,
                                                             counter, out, pairs);
  else
    k_move_energies<false><<<grid, threads, sh.bytes(), st>>>(P, chain, mol, prop, sh, partials,
                                                              counter, out, pairs);
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
