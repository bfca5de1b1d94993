// server.cu -- continuous batching of simulation jobs on one GPU.
//
// The server owns one device arena laid out like a batch pool (rows of all
// resident jobs, pool-absolute indices) with fixed capacities, a slot table
// of chain headers, and three first-fit range allocators (atoms, molecules,
// primary indexes) over the arena.  A round advances every resident job by
// round_steps steps in one launch of the persistent chain kernel over the
// active slots, then (for isobaric jobs) runs the volume phase on the
// active slots' molecules only.  Between rounds finished jobs leave (their
// coordinates and counters go back to the host) and queued jobs enter: their
// rows are copied and initialised (mirrors, chain state, FP64 energy) on a
// second stream while the round in flight runs, in slots and ranges that
// round does not touch.  Admission is FIFO with backfill, limited by free
// slots, free ranges and the HBM budget on the jobs' device footprints.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <vector>

#include "host.h"

using namespace mcgpu;

namespace {

// First-fit allocator over [0, cap) with coalescing frees.
struct RangeAlloc {
  std::map<long long, long long> free_;  // start -> length
  void init(long long cap) {
    free_.clear();
    if (cap > 0) free_[0] = cap;
  }
  long long alloc(long long n) {
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second < n) continue;
      const long long s = it->first, len = it->second;
      free_.erase(it);
      if (len > n) free_[s + n] = len - n;
      return s;
    }
    return -1;
  }
  void release(long long s, long long n) {
    if (n <= 0) return;
    auto it = free_.emplace(s, n).first;
    auto nx = std::next(it);
    if (nx != free_.end() && s + n == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
};

// Device bytes per row element of the arena (see DevPool / server_alloc).
constexpr long long kBytesAtom = 6 * 8 + 16 + 16 + 8 + 16 + 4;          // 108
constexpr long long kBytesMol = 4 + 4 + 8 + 16 + 4 + 16 + 4 + 8 + 8 + 16;  // 88
constexpr long long kBytesPidx = 4 + 16;                                  // 20

struct Job {
  int64_t id = 0;
  HostPool hp;  // the job's rows as chain 0 at offset 0
  int64_t n_steps = 0;
  int npt = 0, vol_mixed = 0;
  double pressure = 0, max_dlnv = 0, lrc_v = 0;
  double *x_out = nullptr, *y_out = nullptr, *z_out = nullptr;
  double t_submit = 0, t_admit = 0;
  long long bytes = 0;
  int slot = -1;
  long long a0 = 0, m0 = 0, p0 = 0;
  int n_atom = 0, n_mol = 0, n_pidx = 0;
};

}  // namespace

struct mcgpu_server {
  mcgpu_ctx* ctx = nullptr;
  mcgpu_server_config cfg{};
  DevPool pool;
  long long cap_atoms = 0, cap_mols = 0, cap_pidx = 0;
  RangeAlloc atoms, mols, pidx;
  std::vector<int> free_slots;
  std::vector<Job*> slot_job;
  std::vector<char> in_round;  // slot was part of the round in flight
  std::deque<Job*> queue;
  std::deque<mcgpu_job_result> done;
  long long in_use = 0;
  int64_t next_id = 1, finished = 0;
  cudaStream_t copy = nullptr;
  cudaEvent_t ev_round = nullptr, ev_copy = nullptr;
  // GPU time of the rounds (chain kernel + volume phase), and the atom pairs
  // the retired jobs evaluated (device-counted)
  cudaEvent_t ev_t0 = nullptr, ev_t1 = nullptr;
  double gpu_s = 0.0;
  long long pairs_done = 0, rounds = 0;
  bool round_in_flight = false, copies_pending = false;
  int gw = 8, grid = 1, smem = 0;
  SmemShape shape{};
  // device scratch
  unsigned* qctr = nullptr;
  int* dlist = nullptr;  // order [slots] | act_slot [slots] | act_m0 [slots] | act_pref [slots+1]
  int* dinit = nullptr;  // per slot: (slot, m0, 0, n_mol) range of a job being initialised
  VolMove* vm = nullptr;
  double2* emol2 = nullptr;
  double2* eabs2 = nullptr;
  double2* vsum = nullptr;
  double2* vsum_abs = nullptr;
  int* vlist = nullptr;        // chains of a re-take (3 * slots + 3)
  // pinned host buffers
  ChainHdr* hmirror = nullptr;
  int* hlist = nullptr;
  char* stage = nullptr;
  size_t stage_cap = 0, stage_off = 0;
  std::chrono::steady_clock::time_point t0;

  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

namespace {

int server_alloc(mcgpu_server* s) {
  mcgpu_ctx* ctx = s->ctx;
  DevPool& dp = s->pool;
  const size_t na = (size_t)s->cap_atoms, nm = (size_t)s->cap_mols, np = (size_t)s->cap_pidx;
  const int nc = s->cfg.max_slots, ml = s->cfg.max_mol_atoms;
  cudaError_t e = cudaSuccess;
  Pool& P = dp.P;
  P.x = dalloc<double>(na, &e); P.y = dalloc<double>(na, &e); P.z = dalloc<double>(na, &e);
  P.sig = dalloc<double>(na, &e); P.eps = dalloc<double>(na, &e); P.q = dalloc<double>(na, &e);
  P.aoff = dalloc<float4>(na, &e); P.aofl = dalloc<float4>(na, &e); P.aeq = dalloc<float2>(na, &e);
  P.atpl = dalloc<float4>(na, &e);
  P.mstart = dalloc<int>(nm, &e); P.mlen = dalloc<int>(nm, &e); P.mpi = dalloc<int2>(nm, &e);
  P.mfix = dalloc<uint4>(nm, &e); P.mrad = dalloc<float>(nm, &e); P.mq = dalloc<float4>(nm, &e);
  P.pidx = dalloc<int>(np, &e); P.ppos = dalloc<float4>(np, &e);
  P.vc_cnt = dalloc<int>(nm, &e); P.vc_start = dalloc<int>(nm, &e);
  P.vc_mol = dalloc<int>(nm, &e); P.vc_of = dalloc<int>(nm, &e);
  P.hdr = dalloc<ChainHdr>(nc, &e);
  P.rb = dalloc<double>((size_t)nc * 3 * ml, &e);
  P.trace = nullptr;
  P.n_chains = nc;
  dp.mol_chain = dalloc<int>(nm, &e);
  dp.atom_mol = dalloc<int>(na, &e);
  dp.emol = dalloc<double>(nm, &e);
  dp.pairs = dalloc<long long>(nm, &e);
  dp.esum = dalloc<double>(nc, &e);
  dp.n_chains = nc;
  dp.n_atom = (int)na;
  dp.n_mol = (int)nm;
  dp.n_pidx = (int)np;
  dp.max_len = ml;
  s->qctr = dalloc<unsigned>(1, &e);
  s->dlist = dalloc<int>(4 * (size_t)nc + 1, &e);
  s->dinit = dalloc<int>(4 * (size_t)nc, &e);
  s->vm = dalloc<VolMove>(nc, &e);
  s->emol2 = dalloc<double2>(nm, &e);
  s->eabs2 = dalloc<double2>(nm, &e);
  s->vsum = dalloc<double2>(nc, &e);
  s->vsum_abs = dalloc<double2>(nc, &e);
  s->vlist = dalloc<int>(3 * (size_t)nc + 3, &e);
  if (e == cudaSuccess) e = cudaMemsetAsync(P.hdr, 0, sizeof(ChainHdr) * nc, ctx->stream);
  if (e == cudaSuccess) e = cudaMallocHost((void**)&s->hmirror, sizeof(ChainHdr) * nc);
  if (e == cudaSuccess) e = cudaMallocHost((void**)&s->hlist, sizeof(int) * (4 * (size_t)nc + 1));
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess)
    return set_err(ctx, MCGPU_ERR_NOMEM, "server arena allocation failed: %s", cudaGetErrorString(e));
  return MCGPU_OK;
}

void server_free(mcgpu_server* s) {
  s->pool.release();
  void* d[] = {s->qctr, s->dlist, s->dinit, s->vm, s->emol2, s->eabs2, s->vsum, s->vsum_abs,
               s->vlist};
  for (void* p : d)
    if (p) cudaFree(p);
  if (s->hmirror) cudaFreeHost(s->hmirror);
  if (s->hlist) cudaFreeHost(s->hlist);
  if (s->stage) cudaFreeHost(s->stage);
  if (s->ev_round) cudaEventDestroy(s->ev_round);
  if (s->ev_t0) cudaEventDestroy(s->ev_t0);
  if (s->ev_t1) cudaEventDestroy(s->ev_t1);
  if (s->ev_copy) cudaEventDestroy(s->ev_copy);
  if (s->copy) cudaStreamDestroy(s->copy);
  for (Job* j : s->slot_job) delete j;
  for (Job* j : s->queue) delete j;
}

// Bytes a job holds on the device while resident.
long long job_bytes(const mcgpu_server* s, int n_atom, int n_mol, int n_pidx) {
  return kBytesAtom * n_atom + kBytesMol * n_mol + kBytesPidx * n_pidx +
         (long long)sizeof(ChainHdr) + 3LL * 8 * s->cfg.max_mol_atoms + 8 + (long long)sizeof(VolMove) + 16;
}

// Pinned staging for `bytes`; earlier staged copies must have completed
// when the buffer wraps or grows.
char* stage_take(mcgpu_server* s, size_t bytes, int* rc) {
  bytes = (bytes + 255) & ~(size_t)255;
  if (s->stage_off + bytes > s->stage_cap) {
    cudaStreamSynchronize(s->copy);
    s->stage_off = 0;
    if (bytes > s->stage_cap) {
      if (s->stage) cudaFreeHost(s->stage);
      s->stage = nullptr;
      size_t cap = std::max<size_t>(bytes, 64u << 20);
      if (cudaMallocHost((void**)&s->stage, cap) != cudaSuccess) {
        s->stage_cap = 0;
        *rc = set_err(s->ctx, MCGPU_ERR_NOMEM, "pinned staging of %zu bytes failed", cap);
        return nullptr;
      }
      s->stage_cap = cap;
    }
  }
  char* p = s->stage + s->stage_off;
  s->stage_off += bytes;
  return p;
}

template <class T>
int stage_copy(mcgpu_server* s, T* dst, const T* src, size_t n) {
  if (n == 0) return MCGPU_OK;
  int rc = MCGPU_OK;
  char* p = stage_take(s, sizeof(T) * n, &rc);
  if (!p) return rc;
  std::memcpy(p, src, sizeof(T) * n);
  CK(s->ctx, cudaMemcpyAsync(dst, p, sizeof(T) * n, cudaMemcpyHostToDevice, s->copy));
  return MCGPU_OK;
}

// Copies job j into its slot and ranges and initialises it (copy stream).
int upload_job(mcgpu_server* s, Job* j) {
  mcgpu_ctx* ctx = s->ctx;
  HostPool& hp = j->hp;
  const int a0 = (int)j->a0, m0 = (int)j->m0, p0 = (int)j->p0, slot = j->slot;
  std::vector<int> mstart(hp.mstart.begin(), hp.mstart.end()), pidx(hp.pidx.begin(), hp.pidx.end()),
      mol_chain(j->n_mol, slot), atom_mol(hp.atom_mol.begin(), hp.atom_mol.end());
  std::vector<int2> mpi(hp.mpi.begin(), hp.mpi.end());
  for (int& v : mstart) v += a0;
  for (int& v : pidx) v += a0;
  for (int& v : atom_mol) v += m0;
  for (int2& v : mpi) v.x += p0;
  ChainHdr h = hp.hdr[0];
  h.atom0 = a0;
  h.mol0 = m0;
  h.pidx0 = p0;
  h.chain_id = hp.hdr[0].chain_id;
  h.step = 0;
  h.step_limit = j->n_steps;
  h.vol_step = 0;
  h.vol_interval = j->npt ? s->cfg.round_steps : 0;
  h.pressure = j->pressure;
  h.max_dlnv = j->max_dlnv;
  h.lrc_v = j->lrc_v;
  h.vol_mixed = j->vol_mixed;
  Pool& P = s->pool.P;
  int rc = MCGPU_OK;
#define SC(dst, vec) \
  if ((rc = stage_copy(s, dst, vec.data(), vec.size()))) return rc
  SC(P.x + a0, hp.x); SC(P.y + a0, hp.y); SC(P.z + a0, hp.z);
  SC(P.sig + a0, hp.sig); SC(P.eps + a0, hp.eps); SC(P.q + a0, hp.q);
  SC(P.aoff + a0, hp.aoff); SC(P.aeq + a0, hp.aeq);
  SC(P.mstart + m0, mstart); SC(P.mlen + m0, hp.mlen); SC(P.mpi + m0, mpi); SC(P.mrad + m0, hp.mrad);
  SC(P.pidx + p0, pidx); SC(s->pool.mol_chain + m0, mol_chain); SC(s->pool.atom_mol + a0, atom_mol);
#undef SC
  if ((rc = stage_copy(s, P.hdr + slot, &h, 1))) return rc;
  const int wpb = 8, n = j->n_mol;
  cudaStream_t st = s->copy;
  k_refresh_mirrors<<<(n + wpb - 1) / wpb, wpb * 32, 0, st>>>(P, s->pool.mol_chain, m0, m0 + n);
  k_chain_init<<<(n + wpb - 1) / wpb, wpb * 32, 0, st>>>(P, s->pool.mol_chain, m0, m0 + n);
  CK(ctx, cudaGetLastError());
  // initial running energy over the job's cell grid (its own molecules,
  // slot and scratch entries only): FP64, or for a job whose volume moves
  // take FP32 pair terms FP32 pairs with their error bound (run_err)
  int* dr = s->dinit + 4 * slot;
  const int rng[4] = {slot, m0, 0, n};
  if ((rc = stage_copy(s, dr, rng, 4))) return rc;
  MolRanges R;
  R.act_slot = dr;
  R.act_m0 = dr + 1;
  R.act_pref = dr + 2;
  R.n_act = 1;
  R.total = n;
  CK(ctx, launch_chain_energy(P, s->pool.mol_chain, 0, s->vm, s->emol2, s->eabs2, s->vsum,
                              s->vsum_abs, st, R, !(j->npt && j->vol_mixed)));
  return MCGPU_OK;
}

// Admits queued jobs that fit, FIFO with backfill.
int admit(mcgpu_server* s) {
  if (s->queue.empty() || s->free_slots.empty()) return MCGPU_OK;
  // the staging buffer restarts once every earlier staged copy has run
  if (cudaEventQuery(s->ev_copy) == cudaSuccess) s->stage_off = 0;
  bool any = false;
  for (auto it = s->queue.begin(); it != s->queue.end() && !s->free_slots.empty();) {
    Job* j = *it;
    if (s->in_use + j->bytes > (long long)s->cfg.hbm_budget_bytes) {
      ++it;
      continue;
    }
    const long long a0 = s->atoms.alloc(j->n_atom);
    const long long m0 = a0 >= 0 ? s->mols.alloc(j->n_mol) : -1;
    const long long p0 = m0 >= 0 ? s->pidx.alloc(j->n_pidx) : -1;
    if (p0 < 0) {
      if (a0 >= 0) s->atoms.release(a0, j->n_atom);
      if (m0 >= 0) s->mols.release(m0, j->n_mol);
      ++it;
      continue;
    }
    j->a0 = a0;
    j->m0 = m0;
    j->p0 = p0;
    j->slot = s->free_slots.back();
    s->free_slots.pop_back();
    s->slot_job[j->slot] = j;
    s->in_use += j->bytes;
    j->t_admit = s->now();
    it = s->queue.erase(it);
    int rc = upload_job(s, j);
    if (rc) return rc;
    any = true;
  }
  if (any) {
    CK(s->ctx, cudaEventRecord(s->ev_copy, s->copy));
    s->copies_pending = true;
  }
  return MCGPU_OK;
}

// Retires the jobs the finished round completed (host header mirror).
int harvest(mcgpu_server* s) {
  mcgpu_ctx* ctx = s->ctx;
  cudaStream_t st = ctx->stream;
  Pool& P = s->pool.P;
  for (int slot = 0; slot < (int)s->slot_job.size(); slot++) {
    Job* j = s->slot_job[slot];
    if (!j || !s->in_round[slot]) continue;  // admitted after that round began
    const ChainHdr& h = s->hmirror[slot];
    if ((int64_t)h.step < j->n_steps && h.error == 0) continue;
    if (j->x_out && j->y_out && j->z_out) {
      const int a0 = (int)j->a0, n = j->n_atom;
      k_chain_export<<<(n + 255) / 256, 256, 0, st>>>(P, s->pool.mol_chain, s->pool.atom_mol, a0,
                                                     a0 + n);
      CK(ctx, cudaGetLastError());
      CK(ctx, cudaMemcpyAsync(j->x_out, P.x + a0, 8 * (size_t)n, cudaMemcpyDeviceToHost, st));
      CK(ctx, cudaMemcpyAsync(j->y_out, P.y + a0, 8 * (size_t)n, cudaMemcpyDeviceToHost, st));
      CK(ctx, cudaMemcpyAsync(j->z_out, P.z + a0, 8 * (size_t)n, cudaMemcpyDeviceToHost, st));
      CK(ctx, cudaStreamSynchronize(st));
    }
    mcgpu_job_result r;
    std::memset(&r, 0, sizeof(r));
    r.job_id = j->id;
    r.energy = h.energy;
    r.steps = (int64_t)h.step;
    r.accepted = h.accepted;
    r.vol_tried = h.vol_tried;
    r.vol_accepted = h.vol_accepted;
    for (int k = 0; k < 3; k++) r.box[k] = h.L[k];
    r.t_submit = j->t_submit;
    r.t_admit = j->t_admit;
    r.t_done = s->now();
    r.footprint_bytes = j->bytes;
    r.error = h.error;
    r.ties = h.ties;
    s->pairs_done += h.pairs;
    s->done.push_back(r);
    s->finished++;
    s->atoms.release(j->a0, j->n_atom);
    s->mols.release(j->m0, j->n_mol);
    s->pidx.release(j->p0, j->n_pidx);
    s->in_use -= j->bytes;
    s->slot_job[slot] = nullptr;
    s->free_slots.push_back(slot);
    delete j;
  }
  return MCGPU_OK;
}

// Launches one round over the resident jobs (compute stream, async).
int launch_round(mcgpu_server* s) {
  mcgpu_ctx* ctx = s->ctx;
  cudaStream_t st = ctx->stream;
  const int nc = s->cfg.max_slots;
  std::vector<int> act;
  for (int slot = 0; slot < nc; slot++) {
    s->in_round[slot] = s->slot_job[slot] != nullptr;
    if (s->slot_job[slot]) act.push_back(slot);
  }
  if (act.empty()) return MCGPU_OK;
  // cost-descending order: screen ~ n_mol, pairs ~ max_len^2
  std::stable_sort(act.begin(), act.end(), [&](int a, int b) {
    const Job* ja = s->slot_job[a];
    const Job* jb = s->slot_job[b];
    return (double)ja->n_mol * (1 + ja->hp.max_len) > (double)jb->n_mol * (1 + jb->hp.max_len);
  });
  int* order = s->hlist;
  int* aslot = s->hlist + nc;
  int* am0 = s->hlist + 2 * nc;
  int* apref = s->hlist + 3 * nc;
  int n_npt = 0, total = 0;
  bool has64 = false, has32 = false;
  for (size_t i = 0; i < act.size(); i++) {
    order[i] = act[i];
    const Job* j = s->slot_job[act[i]];
    if (!j->npt) continue;
    has64 = has64 || !j->vol_mixed;
    has32 = has32 || j->vol_mixed;
    aslot[n_npt] = act[i];
    am0[n_npt] = (int)j->m0;
    apref[n_npt] = total;
    total += j->n_mol;
    n_npt++;
  }
  apref[n_npt] = total;
  CK(ctx, cudaMemcpyAsync(s->dlist, s->hlist, sizeof(int) * (4 * (size_t)nc + 1),
                          cudaMemcpyHostToDevice, st));
  if (s->copies_pending) {
    CK(ctx, cudaStreamWaitEvent(st, s->ev_copy, 0));
    s->copies_pending = false;
  }
  CK(ctx, cudaEventRecord(s->ev_t0, st));
  CK(ctx, cudaMemsetAsync(s->qctr, 0, sizeof(unsigned), st));
  const int need = ((int)act.size() + s->cfg.chains_per_cta - 1) / s->cfg.chains_per_cta;
  const int grid = std::max(1, std::min(need, s->grid));
  if (s->cfg.threads > 256)
    k_chain_steps_wide<<<grid, s->cfg.threads, s->smem, st>>>(s->pool.P, s->cfg.round_steps, s->qctr,
                                                      s->dlist, (int)act.size(), s->gw, s->shape,
                                                      nullptr, 0, 0, s->cfg.lanes_per_molecule);
  else
    k_chain_steps<<<grid, s->cfg.threads, s->smem, st>>>(s->pool.P, s->cfg.round_steps, s->qctr,
                                                      s->dlist, (int)act.size(), s->gw, s->shape,
                                                      nullptr, 0, 0, s->cfg.lanes_per_molecule);
  CK(ctx, cudaGetLastError());
  if (n_npt > 0) {
    MolRanges R;
    R.act_slot = s->dlist + nc;
    R.act_m0 = s->dlist + 2 * nc;
    R.act_pref = s->dlist + 3 * nc;
    R.n_act = n_npt;
    R.total = total;
    CK(ctx, launch_volume_phase(s->pool.P, s->pool.mol_chain, 0, s->vm, s->emol2, s->eabs2,
                                s->vsum, s->vsum_abs, s->vlist, nullptr, 0, 0, st, R, has64,
                                has32));
  }
  CK(ctx, cudaEventRecord(s->ev_t1, st));
  CK(ctx, cudaMemcpyAsync(s->hmirror, s->pool.P.hdr, sizeof(ChainHdr) * nc, cudaMemcpyDeviceToHost, st));
  CK(ctx, cudaEventRecord(s->ev_round, st));
  s->round_in_flight = true;
  return MCGPU_OK;
}

}  // namespace

extern "C" int mcgpu_server_create(mcgpu_ctx* ctx, const mcgpu_server_config* cfg,
                                   mcgpu_server** out) {
  if (!ctx || !cfg || !out) return set_err(ctx, MCGPU_ERR_INVALID, "null argument");
  *out = nullptr;
  mcgpu_server_config c = *cfg;
  if (c.max_slots < 1 || c.max_slots > 4096)
    return set_err(ctx, MCGPU_ERR_INVALID, "max_slots %d outside [1, 4096]", c.max_slots);
  if (c.round_steps < 1) return set_err(ctx, MCGPU_ERR_INVALID, "round_steps %d must be >= 1", c.round_steps);
  if (c.max_mol_atoms < 1 || c.max_mol_atoms > kMaxA)
    return set_err(ctx, MCGPU_ERR_INVALID, "max_mol_atoms %d outside [1, %d]", c.max_mol_atoms, kMaxA);
  if (c.rotation != MCGPU_ROT_EULER && c.rotation != MCGPU_ROT_AXIS)
    return set_err(ctx, MCGPU_ERR_INVALID, "unknown rotation form %d", c.rotation);
  if (c.threads == 0) c.threads = 256;
  if (c.chains_per_cta == 0) c.chains_per_cta = 1;
  if (c.threads < 32 || c.threads > 512 || c.threads % 32 || (c.threads / 32) % c.chains_per_cta)
    return set_err(ctx, MCGPU_ERR_INVALID, "tile %d threads / %d chains per CTA", c.threads,
                   c.chains_per_cta);
  const int lanes = c.lanes_per_molecule;
  if (lanes != 0 && lanes != 1 && lanes != 2 && lanes != 4 && lanes != 8 && lanes != 16 && lanes != 32)
    return set_err(ctx, MCGPU_ERR_INVALID, "lanes per molecule %d", lanes);
  if (c.hbm_budget_bytes == 0) return set_err(ctx, MCGPU_ERR_INVALID, "zero HBM budget");
  CK(ctx, cudaSetDevice(ctx->device));
  mcgpu_server* s = new mcgpu_server();
  s->ctx = ctx;
  s->cfg = c;
  s->t0 = std::chrono::steady_clock::now();
  const long long per_mol = 4 * kBytesAtom + kBytesMol + kBytesPidx;
  s->cap_mols = c.max_molecules > 0 ? c.max_molecules : (long long)(c.hbm_budget_bytes / per_mol);
  s->cap_atoms = c.max_atoms > 0 ? c.max_atoms : 4 * s->cap_mols;
  s->cap_mols = std::min<long long>(std::max<long long>(s->cap_mols, 1), 1LL << 26);
  s->cap_atoms = std::min<long long>(std::max<long long>(s->cap_atoms, 1), 1LL << 30);
  s->cap_pidx = std::min<long long>(2 * s->cap_mols, 1LL << 28);
  s->atoms.init(s->cap_atoms);
  s->mols.init(s->cap_mols);
  s->pidx.init(s->cap_pidx);
  s->slot_job.assign(c.max_slots, nullptr);
  s->in_round.assign(c.max_slots, 0);
  for (int i = c.max_slots - 1; i >= 0; i--) s->free_slots.push_back(i);
  int rc = server_alloc(s);
  cudaError_t e = cudaSuccess;
  if (rc == MCGPU_OK) e = cudaStreamCreateWithFlags(&s->copy, cudaStreamNonBlocking);
  if (rc == MCGPU_OK && e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_round, cudaEventDisableTiming);
  if (rc == MCGPU_OK && e == cudaSuccess) e = cudaEventCreate(&s->ev_t0);
  if (rc == MCGPU_OK && e == cudaSuccess) e = cudaEventCreate(&s->ev_t1);
  if (rc == MCGPU_OK && e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_copy, cudaEventDisableTiming);
  if (rc == MCGPU_OK && e != cudaSuccess)
    rc = set_err(ctx, MCGPU_ERR_CUDA, "server stream/events: %s", cudaGetErrorString(e));
  if (rc) {
    server_free(s);
    delete s;
    return rc;
  }
  s->gw = (c.threads / 32) / c.chains_per_cta;
  s->shape = shape_for(c.max_mol_atoms, s->gw, 2048);
  s->smem = s->shape.bytes() * c.chains_per_cta;
  if (s->smem > 200 * 1024) {
    server_free(s);
    delete s;
    return set_err(ctx, MCGPU_ERR_UNSUPPORTED, "tile needs %d B shared memory", s->smem);
  }
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, c.threads > 256 ? k_chain_steps_wide : k_chain_steps, c.threads, s->smem);
  s->grid = std::max(1, per_sm) * ctx->sm_count;
  *out = s;
  return MCGPU_OK;
}

extern "C" int mcgpu_server_destroy(mcgpu_server* s) {
  if (!s) return MCGPU_OK;
  cudaSetDevice(s->ctx->device);
  cudaStreamSynchronize(s->ctx->stream);
  if (s->copy) cudaStreamSynchronize(s->copy);
  server_free(s);
  delete s;
  return MCGPU_OK;
}

extern "C" int mcgpu_server_submit(mcgpu_server* s, const mcgpu_job_desc* jd, int64_t* job_id) {
  if (!s || !jd || !jd->box) return set_err(s ? s->ctx : nullptr, MCGPU_ERR_INVALID, "null argument");
  mcgpu_ctx* ctx = s->ctx;
  if (jd->n_steps <= 0) return set_err(ctx, MCGPU_ERR_INVALID, "job step count %lld must be > 0",
                                       (long long)jd->n_steps);
  if (jd->npt) {
    if (jd->vol_precision != MCGPU_PREC_FP64 && jd->vol_precision != MCGPU_PREC_MIXED)
      return set_err(ctx, MCGPU_ERR_INVALID, "unknown volume-move precision %d", jd->vol_precision);
    if (!std::isfinite(jd->pressure_atm) || jd->pressure_atm < 0)
      return set_err(ctx, MCGPU_ERR_INVALID, "job pressure %g atm", jd->pressure_atm);
    if (!(jd->max_dlnv > 0 && jd->max_dlnv <= 0.1))
      return set_err(ctx, MCGPU_ERR_INVALID, "job max ln V step %g outside (0, 0.1]", jd->max_dlnv);
    if (!std::isfinite(jd->lrc_v))
      return set_err(ctx, MCGPU_ERR_INVALID, "job lrc_v is not finite");
  }
  Job* j = new Job();
  int rc = append_chain(ctx, j->hp, jd->box, 0, jd->seed, s->cfg.rotation);
  if (rc) {
    delete j;
    return rc;
  }
  j->hp.hdr[0].chain_id = (int)jd->chain_id;
  j->n_atom = jd->box->n_atom;
  j->n_mol = jd->box->n_mol;
  j->n_pidx = jd->box->n_pidx;
  if (j->hp.max_len > s->cfg.max_mol_atoms) {
    delete j;
    return set_err(ctx, MCGPU_ERR_CAPACITY, "job molecule of %d atoms above the server's %d",
                   j->hp.max_len, s->cfg.max_mol_atoms);
  }
  j->bytes = job_bytes(s, j->n_atom, j->n_mol, j->n_pidx);
  if (j->bytes > (long long)s->cfg.hbm_budget_bytes || j->n_atom > s->cap_atoms ||
      j->n_mol > s->cap_mols || j->n_pidx > s->cap_pidx) {
    const long long b = j->bytes;
    delete j;
    return set_err(ctx, MCGPU_ERR_CAPACITY, "job of %lld device bytes can never be admitted", b);
  }
  j->n_steps = jd->n_steps;
  j->npt = jd->npt ? 1 : 0;
  j->pressure = jd->npt ? jd->pressure_atm * kAtmKcal : 0.0;
  j->max_dlnv = jd->npt ? jd->max_dlnv : 0.0;
  j->lrc_v = jd->npt ? jd->lrc_v : 0.0;
  j->vol_mixed = (jd->npt && jd->vol_precision == MCGPU_PREC_MIXED) ? 1 : 0;
  j->x_out = jd->x_out;
  j->y_out = jd->y_out;
  j->z_out = jd->z_out;
  j->id = s->next_id++;
  j->t_submit = s->now();
  s->queue.push_back(j);
  if (job_id) *job_id = j->id;
  return MCGPU_OK;
}

extern "C" int mcgpu_server_step(mcgpu_server* s) {
  if (!s) return set_err(nullptr, MCGPU_ERR_INVALID, "null server");
  mcgpu_ctx* ctx = s->ctx;
  int rc = admit(s);  // into slots the round in flight does not use
  if (rc) return rc;
  if (s->round_in_flight) {
    CK(ctx, cudaEventSynchronize(s->ev_round));
    s->round_in_flight = false;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, s->ev_t0, s->ev_t1) == cudaSuccess) s->gpu_s += 1e-3 * ms;
    s->rounds++;
    rc = harvest(s);
    if (rc) return rc;
    rc = admit(s);
    if (rc) return rc;
  }
  return launch_round(s);
}

extern "C" int mcgpu_server_status(mcgpu_server* s, int* running, int* queued, int64_t* finished,
                                   uint64_t* bytes_in_use) {
  if (!s) return set_err(nullptr, MCGPU_ERR_INVALID, "null server");
  int r = 0;
  for (Job* j : s->slot_job) r += j != nullptr;
  if (running) *running = r;
  if (queued) *queued = (int)s->queue.size();
  if (finished) *finished = s->finished;
  if (bytes_in_use) *bytes_in_use = (uint64_t)s->in_use;
  return MCGPU_OK;
}

extern "C" int mcgpu_server_drain(mcgpu_server* s) {
  if (!s) return set_err(nullptr, MCGPU_ERR_INVALID, "null server");
  for (;;) {
    int running = 0, queued = 0;
    mcgpu_server_status(s, &running, &queued, nullptr, nullptr);
    if (running == 0 && queued == 0 && !s->round_in_flight) return MCGPU_OK;
    int rc = mcgpu_server_step(s);
    if (rc) return rc;
    mcgpu_server_status(s, &running, &queued, nullptr, nullptr);
    if (running == 0 && queued > 0 && !s->round_in_flight)
      return set_err(s->ctx, MCGPU_ERR_CAPACITY, "queued jobs do not fit an empty server");
  }
}

extern "C" int mcgpu_server_results(mcgpu_server* s, mcgpu_job_result* out, int max, int* n) {
  if (!s || !n || (max > 0 && !out)) return set_err(s ? s->ctx : nullptr, MCGPU_ERR_INVALID, "null argument");
  int k = 0;
  while (k < max && !s->done.empty()) {
    out[k++] = s->done.front();
    s->done.pop_front();
  }
  *n = k;
  return MCGPU_OK;
}

extern "C" double mcgpu_server_clock(const mcgpu_server* s) { return s ? s->now() : 0.0; }

extern "C" int mcgpu_server_counters(mcgpu_server* s, int64_t* pairs, double* gpu_seconds,
                                     int64_t* rounds) {
  if (!s) return set_err(nullptr, MCGPU_ERR_INVALID, "null server");
  if (pairs) *pairs = s->pairs_done;
  if (gpu_seconds) *gpu_seconds = s->gpu_s;
  if (rounds) *rounds = s->rounds;
  return MCGPU_OK;
}
