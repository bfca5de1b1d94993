// window.cu -- one chain advanced in windows of K consecutive steps by a
// thread-block cluster of K CTAs (K = 2, 4, 8 or 16), one step of each
// window per CTA.
//
// The reference's loop (Simulation.cpp:219-264) is sequential: step s + 1
// sees the state step s left.  Its moves here come from counter-based draws
// (step index -> move), so the K moves of a window are known before any of
// them is decided.  Every CTA stages all K moves; CTA r evaluates step
// s0 + r against the state at the window's start (FP32 pair terms, the FP64
// re-take inside the guard band -- the one-group kernel's step) and stores
// what it found in every CTA's shared memory (distributed shared memory).
// Every CTA then walks the window in step order.  Step j's result stands
// unless an earlier accepted step i of the window moved the same molecule,
// or moved a molecule whose primaries, before or after step i, come within
// the screen's outer guard radius of step j's molecule at either of its
// placements (the screen of step j could have seen that move).  Such a step
// is staged again if needed and re-evaluated on the current state by every
// CTA alike.  Decisions, coordinates and counters are therefore those of
// the one-group kernel on the same draws; the FP32 pair sums are the
// one-group kernel's too when the CTA has as many warps (same split of the
// candidates over the warps).
//
// Memory: every CTA writes every accepted placement (the same values), and
// a CTA reads the pool only after its own writes of every earlier step.  A
// CTA that runs ahead could only harm a slower one by committing a later
// step while the slower one still reads the state for an earlier step;
// that happens only during a re-evaluation, and a re-evaluated step ends
// with a cluster-wide wait before anyone commits it.  The waits are counts
// stored into every CTA's shared memory (after a release fence) and polled
// in the CTA's own (then an acquire fence), one lane per CTA of the cluster,
// with a time limit: on expiry the chain's error word is set
// and the CTA leaves its loop, so a fault in this protocol ends the launch
// with an error status instead of a stalled GPU.  The only hardware cluster
// barriers are at entry (before any remote store) and at exit (no CTA
// leaves while another may still store into its shared memory); every
// thread passes each of them once.
#include "chain.cuh"
#include "host.h"

namespace mcgpu {

namespace {

// What a CTA found for its step of the window (and what a re-evaluation
// finds): the FP32 totals in double-float, the sum of magnitudes, the
// pairs counted, and the FP64 totals when the decision is taken on them.
struct __align__(16) WinRec {
  float oh, ol, nh, nl, ab;
  int tie;
  long long np;
  double eo, en;
};
static_assert(sizeof(WinRec) == 48, "WinRec layout");

// Wait limit of a cluster-wide wait (ns of the global timer): far above any
// legitimate wait (a step's evaluation, milliseconds at most).
constexpr unsigned long long kWinWaitNs = 4000000000ull;

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

__device__ __forceinline__ unsigned cluster_size() {
  unsigned n;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(n));
  return n;
}

// Hardware cluster barrier (entry and exit only).
__device__ __forceinline__ void cluster_barrier() {
  asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}

// Address of p (this CTA's shared memory) in CTA `rank`'s shared memory.
__device__ __forceinline__ unsigned remote_addr(const void* p, unsigned rank) {
  unsigned a;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;"
               : "=r"(a)
               : "r"((unsigned)__cvta_generic_to_shared(p)), "r"(rank));
  return a;
}

__device__ __forceinline__ void st_remote_u64(unsigned a, unsigned long long v) {
  asm volatile("st.shared::cluster.u64 [%0], %1;" ::"r"(a), "l"(v) : "memory");
}

__device__ __forceinline__ void st_remote_relaxed(unsigned a, unsigned v) {
  asm volatile("st.relaxed.cluster.shared::cluster.u32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned ld_relaxed_cluster(unsigned a) {
  unsigned v;
  asm volatile("ld.relaxed.cluster.shared::cluster.u32 %0, [%1];" : "=r"(v) : "r"(a) : "memory");
  return v;
}

__device__ __forceinline__ void fence_cluster() {
  asm volatile("fence.acq_rel.cluster;" ::: "memory");
}

// Shared memory of the window protocol, after the group's own.
struct WinSmem {
  WinRec* rec;        // [2][K]: the records of the window (two windows in rotation)
  unsigned* flag;     // [K]: barrier count CTA q reached, stored by CTA q
  unsigned* ok;       // [2]: outcome of this CTA's last waits
  char* slots;        // [2][K] staging slots (two windows in rotation)
};

__host__ __device__ inline int win_extra_bytes(const SmemShape& sh, int K) {
  return SmemShape::align16(2 * K * (int)sizeof(WinRec)) + SmemShape::align16(K * 4) + 16 +
         2 * K * sh.ahead_bytes();
}

// Cluster-wide wait number n, lane q of warp 0 serving CTA q: it stores
// rec (if any) into slot rec_at of CTA q's records, fences (release), stores
// the count n into this CTA's flag slot in CTA q, then polls CTA q's slot of
// this CTA's flag row until it reaches n or the limit passes, and fences
// (acquire).  The CTA barrier after it carries what the lanes acquired to
// every thread.  The outcome is the same in every thread of the CTA.
__device__ bool win_wait(const Group& g, const WinSmem& ws, unsigned K, unsigned rank, unsigned n,
                         const WinRec* rec, int rec_at) {
  if (g.tid < 32) {
    const unsigned q = g.tid;
    bool ok = true;
    if (q < K) {
      if (rec) {
        const unsigned a = remote_addr(ws.rec + rec_at, q);
        const unsigned long long* w = (const unsigned long long*)rec;
        for (int k = 0; k < (int)(sizeof(WinRec) / 8); k++) st_remote_u64(a + 8 * k, w[k]);
      }
      fence_cluster();
      st_remote_relaxed(remote_addr(ws.flag + rank, q), n);
      const unsigned a = remote_addr(ws.flag + q, rank);
      const unsigned long long t0 = global_ns();
      unsigned it = 0;
      while (ld_relaxed_cluster(a) < n) {
        if ((++it & 63) == 0 && global_ns() - t0 > kWinWaitNs) {
          ok = false;
          break;
        }
      }
      fence_cluster();
    }
    ok = __all_sync(~0u, ok);
    if (g.tid == 0) ws.ok[n & 1] = ok ? 1u : 0u;
  }
  g.sync();
  return ws.ok[n & 1] != 0;
}

// Step i (slot a, accepted) moved a molecule that step j's screen (slot b)
// could see: a primary pair within the guard band's outer radius for any
// of the four placement pairs, with the screen's own FP32 distance (same
// operands, same order).  The same answer in every lane.
__device__ bool window_near(const StageSlot& a, const StageSlot& b, const ChainHdr& H, int lane) {
  const int na = a.misc[3], nb = b.misc[3];
  bool near = false;
  for (int t = lane; t < na * nb; t += 32) {
    const int ka = t / nb, kb = t - ka * nb;
    const float4 ao = a.p_old[ka], an = a.p_new[ka], bo = b.p_old[kb], bn = b.p_new[kb];
    near = near || r2_screen(bo, ao, H) <= H.cut2_hi || r2_screen(bn, ao, H) <= H.cut2_hi ||
           r2_screen(bo, an, H) <= H.cut2_hi || r2_screen(bn, an, H) <= H.cut2_hi;
  }
  return __any_sync(~0u, near);
}

// The one-group kernel's step evaluation (chain_steps in kernels.cu): FP32
// pair terms over the candidates (the Verlet list when use_list), the FP32
// decision's guard band, and inside it -- or for FP64-pair chains -- both
// placements again with FP64 pairs.  nred counts the group reductions (their
// scratch alternates between two buffers).
__device__ void window_eval(const Pool& P, const ChainHdr& H, const Group& g, const GroupSmem& ss,
                            const MovedInfo& mi, const float4* pcache, bool use_list, int T,
                            float u, int& nred, WinRec& x) {
  const int lane = g.tid & 31, w = g.warp(), nw = g.nwarps();
  AccFF acc = {0.f, 0.f, 0.f, 0.f, 0.f, 0};
  const bool f64all = H.fp64_pairs != 0;
  if (f64all) {
  } else if (use_list) {
    warp_eval_chain(P, H, ss, mi, pcache, 0, P.nl_cnt[mi.mol], w, nw, lane, T, acc,
                    P.nl + (size_t)mi.mol * P.nl_stride);
  } else {
    warp_eval_chain(P, H, ss, mi, pcache, H.mol0, H.mol0 + H.n_mol, w, nw, lane, T, acc);
  }
  group_reduce_ff(g, ss, acc, nred++ & 1);
  const float de_f = __fadd_rn(__fsub_rn(acc.nh, acc.oh), __fsub_rn(acc.nl, acc.ol));
  const float bound = (float)kTieRel * acc.ab + 2.4e-7f * (fabsf(acc.nh) + fabsf(acc.oh)) + 1e-9f;
  const float pf = expf(-fmaxf(de_f, 0.f) * H.kTinvf);
  const int tie = f64all ||
                  ((de_f >= -bound) && (fabsf(pf - u) <= pf * (1.5f * bound * H.kTinvf) + 1e-6f));
  x.oh = acc.oh;
  x.ol = acc.ol;
  x.nh = acc.nh;
  x.nl = acc.nl;
  x.ab = acc.ab;
  x.np = acc.np;
  x.tie = tie;
  x.eo = 0.0;
  x.en = 0.0;
  if (tie) {
    if (w == 0) stage_chain_f64(P, H, ss, mi, lane);
    g.sync();
    double eo = 0.0, en = 0.0, ab2 = 0.0;
    long long np2 = 0;
    if (use_list)
      warp_eval_chain64(P, H, ss, mi, pcache, 0, P.nl_cnt[mi.mol], w, nw, lane, T, eo, en,
                        P.nl + (size_t)mi.mol * P.nl_stride);
    else
      warp_eval_chain64(P, H, ss, mi, pcache, H.mol0, H.mol0 + H.n_mol, w, nw, lane, T, eo, en);
    group_reduce(g, ss, eo, en, ab2, np2, nred++ & 1);
    x.eo = eo;
    x.en = en;
  }
}

}  // namespace

// One cluster of K CTAs per chain task (task k runs chain order[k]; cluster
// c takes tasks c, c + clusters, ...), one group of all the CTA's warps per
// CTA; n_steps steps per chain in windows of K.  trace, trace_off,
// trace_stride and lanes_cap as in chain_steps.
__global__ void __launch_bounds__(512, 1)
    k_chain_window(Pool P, int n_steps, const int* order, int n_tasks, SmemShape shape,
                   mcgpu_trace* trace, int trace_off, int trace_stride, int lanes_cap) {
  extern __shared__ __align__(16) char smem[];
  const unsigned K = cluster_size(), rank = cluster_rank();
  const int n_cl = (int)(gridDim.x / K), cid = (int)(blockIdx.x / K);
  const Group g{(int)threadIdx.x, (int)blockDim.x, 1};
  GroupSmem s = shape.carve(smem);
  WinSmem ws;
  {
    char* p = smem + shape.bytes();
    ws.rec = (WinRec*)p;
    p += SmemShape::align16(2 * K * (int)sizeof(WinRec));
    ws.flag = (unsigned*)p;
    p += SmemShape::align16(K * 4);
    ws.ok = (unsigned*)p;
    p += 16;
    ws.slots = p;
  }
  const int sbytes = shape.ahead_bytes();
  auto slot = [&](int par, int j) { return shape.ahead_slot(ws.slots + (par * (int)K + j) * sbytes); };
  const int lane = threadIdx.x & 31, w = g.warp(), nw = g.nwarps();
  for (int q = g.tid; q < (int)K; q += g.nthreads) ws.flag[q] = 0u;
  cluster_barrier();
  unsigned nbar = 0;
  bool alive = true;
  for (int task = cid; task < n_tasks && alive; task += n_cl) {
    const int c = order[task];
    ChainHdr* Hp = P.hdr + c;
    const ChainHdr& H = *Hp;
    float4* pcache = (s.pc && H.simple_prim && H.n_mol <= shape.cache_n) ? s.pc : nullptr;
    if (pcache)
      for (int i = g.tid; i < H.n_mol; i += g.nthreads) pcache[i] = P.ppos[H.pidx0 + i];
    if (H.uniform)
      for (int i = g.tid; i < H.ulen; i += g.nthreads) s.teq[i] = P.aeq[H.atom0 + i];
    g.sync();
    if (g.tid == 0) Hp->ljmask = uniform_lj_mask(P, H, s.teq);  // the same value in every CTA
    const bool lead = rank == 0 && g.tid == 0;
    int full_scans = 0, ties = 0, redo = 0;
    float de_h = 0.f, de_l = 0.f, err_h = 0.f, err_l = 0.f;
    long long acc_n = 0, npairs = 0;
    const unsigned long long step0 = H.step;
    bool nl_ok = H.nl_on && H.nl_valid;
    const int T = lanes_cap > 0 ? min(lanes_cap, H.tpm)
                                : ((H.uniform && H.ulen <= 4 && !H.precise) ? 1 : H.tpm);
    MoveF* props = (MoveF*)s.props;
    int my_steps = n_steps;
    if (H.step_limit > 0)
      my_steps = (int)max(0LL, min((long long)n_steps, H.step_limit - (long long)step0));
    int nred = 0;
    for (int s0 = 0; s0 < my_steps; s0 += (int)K) {
      const int nst = min((int)K, my_steps - s0), par = (s0 / (int)K) & 1;
      // draws 32 steps at a time (K divides 32, so a window never straddles)
      if ((s0 & 31) == 0) {
        if (w == 0) {
          if (s0 + lane < my_steps)
            props[lane] = draw_move_f32(H.seed, H.chain_id, step0 + s0 + lane, H.n_mol,
                                        P.mlen + H.mol0, (float)H.max_t, (float)H.max_r,
                                        H.rot_mode);
          __syncwarp();
        }
        g.sync();
      }
      // warp j stages step s0 + j (slots of the other parity may still be
      // read by warps finishing the previous window)
      if (w < nst) stage_chain(P, H, props[(s0 + w) & 31], slot(par, w), pcache, lane);
      g.sync();
      const bool nl_ok0 = nl_ok;
      WinRec x = {};
      if ((int)rank < nst) {
        const GroupSmem ss = with_slot(s, slot(par, rank));
        const MovedInfo mi = load_moved(ss);
        window_eval(P, H, g, ss, mi, pcache, nl_ok0 && ss.misc[kMiscNlTrial] != 0, T,
                    __int_as_float(ss.misc[kMiscU]), nred, x);
      }
      if (!win_wait(g, ws, K, rank, ++nbar, &x, par * (int)K + (int)rank)) {
        alive = false;
        break;
      }
      unsigned accm = 0;
      for (int j = 0; j < nst; j++) {
        const StageSlot tj = slot(par, j);
        const GroupSmem ss = with_slot(s, tj);
        MovedInfo mi = load_moved(ss);
        bool same = false, near = false;
        for (int i = 0; i < j; i++) {
          if (!((accm >> i) & 1u)) continue;
          const StageSlot ti = slot(par, i);
          if (ti.misc[0] == mi.mol)
            same = true;
          else if (!near)
            near = window_near(ti, tj, H, lane);
        }
        WinRec xj;
        bool listed;
        if (same || near) {
          if (same) {
            // the move was staged from rows an earlier step of the window
            // changed: stage it again once every warp is done reading it
            g.sync();
            if (w == 0) stage_chain(P, H, props[(s0 + j) & 31], tj, pcache, lane);
            g.sync();
            mi = load_moved(ss);
          }
          listed = nl_ok && ss.misc[kMiscNlTrial] != 0;
          window_eval(P, H, g, ss, mi, pcache, listed, T, __int_as_float(ss.misc[kMiscU]), nred,
                      xj);
          // nobody commits step j (or a later one) while a CTA still reads
          // the state for it
          if (!win_wait(g, ws, K, rank, ++nbar, nullptr, 0)) {
            alive = false;
            break;
          }
          redo++;
        } else {
          xj = ws.rec[par * (int)K + j];
          listed = nl_ok0 && ss.misc[kMiscNlTrial] != 0;
        }
        const float u = __int_as_float(ss.misc[kMiscU]);
        const float de_f = __fadd_rn(__fsub_rn(xj.nh, xj.oh), __fsub_rn(xj.nl, xj.ol));
        const float bound =
            (float)kTieRel * xj.ab + 2.4e-7f * (fabsf(xj.nh) + fabsf(xj.oh)) + 1e-9f;
        int ok;
        if (xj.tie) {
          const double d64 = xj.en - xj.eo;
          ok = (d64 < 0) || (exp(-d64 / H.kT) >= (double)u);
        } else {
          const float pf = expf(-fmaxf(de_f, 0.f) * H.kTinvf);
          ok = (de_f < 0.f) || (pf >= u);
        }
        if (ok) {
          commit_chain(P, H, ss, mi, pcache, lane);
          accm |= 1u << j;
        }
        __syncwarp();
        if (ok && !ss.misc[kMiscNlTrial]) nl_ok = false;
        if (lead) {
          if (ok) {
            if (xj.tie) {
              const double d64 = xj.en - xj.eo;
              const float dh = (float)d64;
              ff_add2(de_h, de_l, dh, (float)(d64 - (double)dh));
              ff_add(err_h, err_l, 1e-12f * xj.ab);
            } else {
              ff_add2(de_h, de_l, xj.nh, xj.nl);
              ff_add2(de_h, de_l, -xj.oh, -xj.ol);
              ff_add(err_h, err_l, bound);
            }
            acc_n++;
          }
          if (H.nl_on && !listed) full_scans++;
          npairs += xj.np;
          ties += xj.tie;
          if (trace) {
            double e_old = xj.eo, e_new = xj.en;
            if (!xj.tie) {
              e_old = (double)xj.oh + (double)xj.ol;
              e_new = (double)xj.nh + (double)xj.nl;
            }
            mcgpu_trace t;
            t.mol = mi.mol - H.mol0;
            t.accepted = ok;
            t.e_old = e_old;
            t.e_new = e_new;
            t.de = e_new - e_old;
            t.u = (double)u;
            t.fp64 = xj.tie;
            t.pad0 = 0;
            trace[(size_t)c * trace_stride + trace_off + s0 + j] = t;
          }
        }
      }
      if (!alive) break;
    }
    if (!alive) {
      if (g.tid == 0) Hp->error = kErrWindowSync;
      break;
    }
    if (lead) {
      Hp->energy = H.energy + ((double)de_h + (double)de_l);
      Hp->run_err += (double)err_h + (double)err_l;
      Hp->step = step0 + my_steps;
      Hp->accepted += acc_n;
      Hp->pairs += npairs;
      Hp->ties += ties;
      Hp->win_redo += redo;
      if (H.nl_on) {
        Hp->nl_valid = nl_ok ? 1 : 0;
        Hp->nl_full += full_scans;
      }
    }
    g.sync();
  }
  cluster_barrier();
}

int window_smem_bytes(const SmemShape& sh, int K) { return sh.bytes() + win_extra_bytes(sh, K); }

cudaError_t window_init() {
  const cudaError_t e = cudaFuncSetAttribute(
      k_chain_window, cudaFuncAttributeMaxDynamicSharedMemorySize, kWindowSmemMax);
  if (e != cudaSuccess) return e;
  // clusters of 16 CTAs are beyond the portable size of 8; where the device
  // refuses them, window_max_clusters reports none and the setters refuse
  // the window
  if (cudaFuncSetAttribute(k_chain_window, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
      cudaSuccess)
    cudaGetLastError();
  return cudaSuccess;
}

int window_max_clusters(int K, int threads, int smem) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(K, 1, 1);
  cfg.blockDim = dim3(threads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = K;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, k_chain_window, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

cudaError_t launch_chain_window(int K, int n_clusters, int threads, int smem, cudaStream_t st,
                                const Pool& P, int n_steps, const int* order, int n_tasks,
                                SmemShape sh, mcgpu_trace* trace, int trace_off, int trace_stride,
                                int lanes_cap) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(K * n_clusters, 1, 1);
  cfg.blockDim = dim3(threads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = K;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_chain_window, P, n_steps, order, n_tasks, sh, trace, trace_off,
                            trace_stride, lanes_cap);
}

}  // namespace mcgpu
