// abi.cu -- host side of the C ABI declared in include/mcgpu_gb300.h.
//
// A box (plain single chain) and a batch (many chains) are both a device
// "pool": one allocation per row, chains concatenated, per-chain headers.
// Kernels live in kernels.cu; this file validates inputs, lays out the pool,
// launches, and turns CUDA failures into status codes.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "host.h"
#include "intra.h"


using namespace mcgpu;

// ---- errors ------------------------------------------------------------------

static thread_local std::string g_err;


int set_err(mcgpu_ctx* ctx, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  if (ctx) ctx->err = buf;
  return code;
}

namespace mcgpu {
// Error text of context-free entry points, read by mcgpu_last_error(NULL, ...).
void note_process_error(const char* msg) { g_err = msg; }
}  // namespace mcgpu


// ---- pool ----------------------------------------------------------------------

namespace mcgpu {

// Sizes of descriptor d (chain c), validated: 0 or an error code with err.
static int chain_sizes(const mcgpu_box_desc* d, int c, std::string* err) {
  char buf[512];
  if (!d) {
    *err = "null box descriptor";
    return MCGPU_ERR_INVALID;
  }
  if (d->n_mol <= 0 || d->n_atom <= 0 || d->n_pidx <= 0) {
    snprintf(buf, sizeof(buf), "chain %d: empty box (n_mol=%d n_atom=%d n_pidx=%d)", c, d->n_mol,
             d->n_atom, d->n_pidx);
    *err = buf;
    return MCGPU_ERR_INVALID;
  }
  return MCGPU_OK;
}

// Validates descriptor d (chain c) and writes it into the host pool at
// atom0 / mol0 / pidx0 and header slot `slot` (the rows are sized already).
// On failure returns the error code with its text in err.
static int fill_chain(HostPool& hp, const mcgpu_box_desc* d, int c, int slot, int atom0, int mol0,
                      int pidx0, unsigned long long seed, int rot_mode, std::string* err) {
  char ebuf[512];
  auto fail = [&](int code, const char* fmt, auto... args) {
    snprintf(ebuf, sizeof(ebuf), fmt, args...);
    *err = ebuf;
    return code;
  };
  if (!d->x || !d->y || !d->z || !d->sigma || !d->epsilon || !d->charge || !d->mol_start ||
      !d->mol_len || !d->mol_pidx_start || !d->mol_pidx_count || !d->pidx)
    return fail(MCGPU_ERR_INVALID, "chain %d: null row pointer", c);
  for (int k = 0; k < 3; k++)
    if (!(d->size[k] > 0) || !std::isfinite(d->size[k]))
      return fail(MCGPU_ERR_INVALID, "chain %d: box edge %d is %g", c, k, d->size[k]);
  if (!(d->cutoff > 0) || !(d->temperature > 0))
    return fail(MCGPU_ERR_INVALID, "chain %d: cutoff %g / temperature %g must be > 0", c,
                   d->cutoff, d->temperature);
  for (int a = 0; a < d->n_atom; a++) {
    const size_t at = (size_t)atom0 + a;
    hp.x[at] = d->x[a];
    hp.y[at] = d->y[a];
    hp.z[at] = d->z[a];
    hp.sig[at] = d->sigma[a];
    hp.eps[at] = d->epsilon[a];
    hp.q[at] = d->charge[a];
    if (!std::isfinite(d->x[a]) || !std::isfinite(d->y[a]) || !std::isfinite(d->z[a]))
      return fail(MCGPU_ERR_INVALID, "chain %d: non-finite coordinate at atom %d", c, a);
    const bool active = d->sigma[a] >= 0 && d->epsilon[a] >= 0;  // BruteForceStep.cpp:64-65
    hp.aoff[at] = make_float4(0.f, 0.f, 0.f, active ? (float)d->sigma[a] : 0.f);
    hp.aeq[at] = active ? make_float2((float)(2.0 * std::sqrt(std::fabs(d->epsilon[a]))),
                                      (float)(d->charge[a] * std::sqrt(kCoulomb)))
                        : make_float2(0.f, 0.f);
  }
  int max_len = 0;
  double max_rad = 0, max_prad = 0;
  bool simple = d->n_pidx == d->n_mol;
  bool uniform = simple;
  int u_len = -1, u_act = -1, u_prim = -1;
  float u_mrad = 0.f;
  for (int m = 0; m < d->n_mol; m++) {
    const int s = d->mol_start[m], len = d->mol_len[m];
    const int ps = d->mol_pidx_start[m], pc = d->mol_pidx_count[m];
    if (len < 1 || len > kMaxA)
      return fail(MCGPU_ERR_UNSUPPORTED, "chain %d molecule %d: %d atoms (limit %d)", c, m,
                     len, kMaxA);
    if (s < 0 || s + len > d->n_atom)
      return fail(MCGPU_ERR_INVALID, "chain %d molecule %d: atoms [%d,%d) outside [0,%d)",
                     c, m, s, s + len, d->n_atom);
    if (pc < 1 || pc > kMaxP)
      return fail(MCGPU_ERR_UNSUPPORTED, "chain %d molecule %d: %d primary indexes (1..%d)",
                     c, m, pc, kMaxP);
    if (ps < 0 || ps + pc > d->n_pidx)
      return fail(MCGPU_ERR_INVALID, "chain %d molecule %d: primary range outside pidx", c,
                     m);
    int act = 0;
    for (int a = s; a < s + len; a++) act += (d->sigma[a] >= 0 && d->epsilon[a] >= 0);
    for (int k = ps; k < ps + pc; k++) {
      const int p = d->pidx[k];
      if (p < s || p >= s + len)
        return fail(MCGPU_ERR_INVALID,
                       "chain %d molecule %d: primary index %d outside its atoms", c, m, p);
    }
    const int an = d->pidx[ps];
    double rad = 0;
    for (int a = s; a < s + len; a++) {
      const double dx = d->x[a] - d->x[an], dy = d->y[a] - d->y[an], dz = d->z[a] - d->z[an];
      rad = std::max(rad, std::sqrt(dx * dx + dy * dy + dz * dz));
    }
    for (int k = ps; k < ps + pc; k++) {
      const int p = d->pidx[k];
      const double dx = d->x[p] - d->x[an], dy = d->y[p] - d->y[an], dz = d->z[p] - d->z[an];
      max_prad = std::max(max_prad, std::sqrt(dx * dx + dy * dy + dz * dz));
    }
    max_rad = std::max(max_rad, rad);
    max_len = std::max(max_len, len);
    const size_t mo = (size_t)mol0 + m;
    hp.mstart[mo] = atom0 + s;
    hp.mlen[mo] = len | (act << 8);
    hp.mpi[mo] = make_int2(pidx0 + ps, pc);
    hp.mrad[mo] = (float)(rad * (1 + 1e-6) + 1e-4);
    hp.mol_chain[mo] = c;
    if (ps != m || pc != 1) simple = false;
    if (m == 0) {
      u_len = len;
      u_act = act;
      u_prim = an - s;
    }
    if (!simple || s != m * u_len || len != u_len || act != u_act || an - s != u_prim)
      uniform = false;
    // the same species: identical parameters slot by slot
    for (int k = 0; uniform && k < len; k++)
      if (d->sigma[s + k] != d->sigma[k] || d->epsilon[s + k] != d->epsilon[k] ||
          d->charge[s + k] != d->charge[k])
        uniform = false;
    u_mrad = std::max(u_mrad, hp.mrad[mo]);
  }
  for (int a = 0; a < d->n_atom; a++) hp.atom_mol[(size_t)atom0 + a] = -1;
  for (int m = 0; m < d->n_mol; m++)
    for (int a = d->mol_start[m]; a < d->mol_start[m] + d->mol_len[m]; a++)
      hp.atom_mol[atom0 + a] = mol0 + m;
  for (int a = 0; a < d->n_atom; a++)
    if (hp.atom_mol[atom0 + a] < 0)
      return fail(MCGPU_ERR_INVALID, "chain %d: atom %d belongs to no molecule", c, a);
  const double Lmin = std::min(d->size[0], std::min(d->size[1], d->size[2]));
  if (max_rad >= 0.25 * Lmin)
    return fail(MCGPU_ERR_UNSUPPORTED,
                   "chain %d: molecule radius %.3f A reaches a quarter of the box edge %.3f A", c,
                   max_rad, Lmin);
  for (int k = 0; k < d->n_pidx; k++) hp.pidx[(size_t)pidx0 + k] = atom0 + d->pidx[k];

  ChainHdr h;
  std::memset(&h, 0, sizeof(h));
  h.atom0 = atom0;
  h.mol0 = mol0;
  h.pidx0 = pidx0;
  h.n_mol = d->n_mol;
  h.n_atom = d->n_atom;
  h.n_pidx = d->n_pidx;
  h.max_len = max_len;
  int T = 1;
  while (T < max_len && T < 32) T <<= 1;
  h.tpm = T;
  h.rot_mode = rot_mode;
  h.chain_id = (int)c;
  h.simple_prim = simple ? 1 : 0;
  h.uniform = uniform ? 1 : 0;
  h.ulen = u_len;
  h.uact = u_act;
  h.uprim = u_prim;
  h.umrad = u_mrad;
  h.precise = max_len >= 8 ? 1 : 0;
  const double rc = d->cutoff;
  h.cutoff = rc;
  hdr_set_box(h, d->size);
  h.kTinvf = (float)(1.0 / (d->temperature * kBoltz));
  h.rad_max = (float)max_rad;
  h.prad = (float)max_prad;
  h.kT = d->temperature * kBoltz;  // SimBoxBuilder.cpp:29
  h.max_t = d->max_translate;
  h.max_r = d->max_rotate;
  h.seed = seed;
  hp.hdr[slot] = h;
  return MCGPU_OK;
}

// Validates one descriptor and appends it as chain `c` of the host pool.
int append_chain(mcgpu_ctx* ctx, HostPool& hp, const mcgpu_box_desc* d, int c,
                 unsigned long long seed, int rot_mode) {
  std::string err;
  int rc = chain_sizes(d, c, &err);
  if (rc) return set_err(ctx, rc, "%s", err.c_str());
  const size_t atom0 = hp.x.size(), mol0 = hp.mstart.size(), pidx0 = hp.pidx.size();
  if (atom0 + d->n_atom > (1ull << 30) || mol0 + d->n_mol > (1ull << 26) ||
      pidx0 + d->n_pidx > (1ull << 30))
    return set_err(ctx, MCGPU_ERR_UNSUPPORTED, "pool too large");
  const size_t slot = hp.hdr.size();
  hp.resize(atom0 + d->n_atom, mol0 + d->n_mol, pidx0 + d->n_pidx, slot + 1);
  rc = fill_chain(hp, d, c, (int)slot, (int)atom0, (int)mol0, (int)pidx0, seed, rot_mode, &err);
  if (rc) {
    hp.resize(atom0, mol0, pidx0, slot);
    return set_err(ctx, rc, "%s", err.c_str());
  }
  hp.max_len = std::max(hp.max_len, hp.hdr[slot].max_len);
  return MCGPU_OK;
}

// The host pool of n chains: sizes and offsets first, then the chains
// filled in parallel on the host's cores (one thread per chain, so each
// chain's checks run in their usual order). The error reported is the one a
// chain-by-chain build meets first: the lowest chain that fails.
int build_pool(mcgpu_ctx* ctx, HostPool& hp, const mcgpu_box_desc* descs, int n,
               const uint64_t* seeds, int rot_mode) {
  std::vector<size_t> a0(n + 1, 0), m0(n + 1, 0), p0(n + 1, 0);
  std::string size_err;
  int size_rc = MCGPU_OK, n_ok = n;
  for (int c = 0; c < n; c++) {
    size_rc = chain_sizes(&descs[c], c, &size_err);
    if (!size_rc) {
      a0[c + 1] = a0[c] + descs[c].n_atom;
      m0[c + 1] = m0[c] + descs[c].n_mol;
      p0[c + 1] = p0[c] + descs[c].n_pidx;
      if (a0[c + 1] > (1ull << 30) || m0[c + 1] > (1ull << 26) || p0[c + 1] > (1ull << 30)) {
        size_rc = MCGPU_ERR_UNSUPPORTED;
        size_err = "pool too large";
      }
    }
    if (size_rc) {
      n_ok = c;
      break;
    }
  }
  hp.resize(a0[n_ok], m0[n_ok], p0[n_ok], (size_t)n_ok);
  std::vector<int> codes(n_ok, MCGPU_OK);
  std::vector<std::string> errs(n_ok);
  std::atomic<int> next{0};
  auto work = [&]() {
    for (int c = next++; c < n_ok; c = next++)
      codes[c] = fill_chain(hp, &descs[c], c, c, (int)a0[c], (int)m0[c], (int)p0[c], seeds[c],
                            rot_mode, &errs[c]);
  };
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t nt = std::min<size_t>({(size_t)hw, (size_t)16, (size_t)std::max(n_ok, 1),
                                      a0[n_ok] / 20000 + 1});
  std::vector<std::thread> pool;
  for (size_t t = 1; t < nt; t++) {
    try {
      pool.emplace_back(work);
    } catch (const std::system_error&) {
      break;  // fewer helpers; the calling thread takes what is left
    }
  }
  work();
  for (std::thread& th : pool) th.join();
  for (int c = 0; c < n_ok; c++)
    if (codes[c]) return set_err(ctx, codes[c], "%s", errs[c].c_str());
  if (size_rc) return set_err(ctx, size_rc, "%s", size_err.c_str());
  for (int c = 0; c < n; c++) hp.max_len = std::max(hp.max_len, hp.hdr[c].max_len);
  return MCGPU_OK;
}

int upload_pool(mcgpu_ctx* ctx, HostPool& hp, DevPool& dp) {
  cudaError_t e = cudaSuccess;
  const size_t na = hp.x.size(), nm = hp.mstart.size(), np = hp.pidx.size(), nc = hp.hdr.size();
  dp.n_chains = (int)nc;
  dp.n_atom = (int)na;
  dp.n_mol = (int)nm;
  dp.n_pidx = (int)np;
  dp.max_len = hp.max_len;
  Pool& P = dp.P;
  P.x = dalloc<double>(na, &e); P.y = dalloc<double>(na, &e); P.z = dalloc<double>(na, &e);
  P.sig = dalloc<double>(na, &e); P.eps = dalloc<double>(na, &e); P.q = dalloc<double>(na, &e);
  P.aoff = dalloc<float4>(na, &e); P.aeq = dalloc<float2>(na, &e);
  P.aofl = dalloc<float4>(na, &e); P.blend = dalloc<double2>(na, &e);
  P.mstart = dalloc<int>(nm, &e); P.mlen = dalloc<int>(nm, &e); P.mpi = dalloc<int2>(nm, &e);
  P.mfix = dalloc<uint4>(nm, &e); P.mrad = dalloc<float>(nm, &e);
  P.mq = dalloc<float4>(nm, &e); P.atpl = dalloc<float4>(na, &e);
  P.pidx = dalloc<int>(np, &e); P.ppos = dalloc<float4>(np, &e);
  P.hdr = dalloc<ChainHdr>(nc, &e);
  P.rb = dalloc<double>(nc * 3 * (size_t)hp.max_len, &e);
  P.trace = nullptr;
  P.n_chains = (int)nc;
  dp.mol_chain = dalloc<int>(nm, &e);
  dp.atom_mol = dalloc<int>(na, &e);
  dp.emol = dalloc<double>(nm, &e);
  dp.pairs = dalloc<long long>(nm, &e);
  dp.esum = dalloc<double>(nc, &e);
  if (e != cudaSuccess) {
    dp.release();
    return set_err(ctx, MCGPU_ERR_NOMEM, "device allocation failed: %s", cudaGetErrorString(e));
  }
  cudaStream_t st = ctx->stream;
#define UP(dst, src) CK(ctx, cudaMemcpyAsync(dst, src.data(), sizeof(src[0]) * src.size(), cudaMemcpyHostToDevice, st))
  UP(P.x, hp.x); UP(P.y, hp.y); UP(P.z, hp.z);
  UP(P.sig, hp.sig); UP(P.eps, hp.eps); UP(P.q, hp.q);
  UP(P.aoff, hp.aoff); UP(P.aeq, hp.aeq);
  UP(P.mstart, hp.mstart); UP(P.mlen, hp.mlen); UP(P.mpi, hp.mpi); UP(P.mrad, hp.mrad);
  UP(P.pidx, hp.pidx); UP(P.hdr, hp.hdr); UP(dp.mol_chain, hp.mol_chain);
  UP(dp.atom_mol, hp.atom_mol);
#undef UP
  const int wpb = 8;
  k_refresh_mirrors<<<(int)((nm + wpb - 1) / wpb), wpb * 32, 0, st>>>(P, dp.mol_chain, 0, (int)nm);
  CK(ctx, cudaGetLastError());
  if (na > 0) k_blend_rows<<<(int)((na + 255) / 256), 256, 0, st>>>(P, (int)na);
  CK(ctx, cudaGetLastError());
  CK(ctx, cudaStreamSynchronize(st));
  dp.hdr.assign(hp.hdr.begin(), hp.hdr.end());
  dp.mstart.assign(hp.mstart.begin(), hp.mstart.end());
  dp.mlen.assign(hp.mlen.begin(), hp.mlen.end());
  return MCGPU_OK;
}

SmemShape shape_for(int max_len, int nwarps, int cache_n) {
  SmemShape s;
  s.maxA = std::max(max_len, 1);
  s.nwarps = nwarps;
  s.cache_n = cache_n;
  return s;
}

int pool_cache_n(const DevPool& dp) {
  int n = 0;
  for (const ChainHdr& h : dp.hdr) {
    if (!h.simple_prim) return 0;
    n = std::max(n, h.n_mol);
  }
  return n <= kCacheMax ? n : 0;
}

// Chain state from the FP64 rows (snaps the rows to it).
int pool_chain_init(mcgpu_ctx* ctx, DevPool& dp, cudaStream_t st) {
  const int wpb = 8;
  k_chain_init<<<(dp.n_mol + wpb - 1) / wpb, wpb * 32, 0, st>>>(dp.P, dp.mol_chain, 0, dp.n_mol);
  CK(ctx, cudaGetLastError());
  return MCGPU_OK;
}

// FP64 rows from the chain state.
int pool_chain_export(mcgpu_ctx* ctx, DevPool& dp, cudaStream_t st) {
  k_chain_export<<<(dp.n_atom + 255) / 256, 256, 0, st>>>(dp.P, dp.mol_chain, dp.atom_mol, 0,
                                                         dp.n_atom);
  CK(ctx, cudaGetLastError());
  return MCGPU_OK;
}

int pool_set_verlet(mcgpu_ctx* ctx, DevPool& dp, double skin, cudaStream_t st) {
  const int nc = dp.n_chains;
  std::vector<NlCfg> cfg(nc);
  int cells = 0, max_cells = 0;
  long long stride = 0;
  for (int c = 0; c < nc; c++) {
    const ChainHdr& h = dp.hdr[c];
    NlCfg& f = cfg[c];
    std::memset(&f, 0, sizeof(f));
    if (skin <= 0) continue;
    const double rl = h.cutoff + skin + 2.0 * h.prad;
    int cap = 1;
    for (int k = 0; k < 3; k++) cap *= (int)std::floor(1.25 * h.L[k] / rl) + 1;
    f.on = 1;
    f.cell0 = cells;
    f.cell_cap = cap;
    f.rlist = (float)rl;
    f.r2 = (float)((rl + 1e-2) * (rl + 1e-2));
    const double hs = std::max(0.5 * skin - 1e-2, 0.0);
    f.half2 = (float)(hs * hs);
    cells += cap;
    max_cells = std::max(max_cells, cap);
    const double rho = h.n_mol / (h.L[0] * h.L[1] * h.L[2]);
    const double est = rho * 4.18879020478639 * std::pow(rl + 1e-2, 3);
    stride = std::max<long long>(stride, std::min<long long>((long long)(2 * est) + 64, h.n_mol));
  }
  stride = (stride + 31) & ~31LL;
  Pool& P = dp.P;
  void* old[] = {P.nl, P.nl_cnt, P.pbuild, P.mcell, P.cell_cnt, P.cell_start, P.cell_mol};
  for (void* p : old)
    if (p) cudaFree(p);
  P.nl = nullptr; P.nl_cnt = nullptr; P.pbuild = nullptr; P.mcell = nullptr;
  P.cell_cnt = nullptr; P.cell_start = nullptr; P.cell_mol = nullptr;
  P.nl_stride = 0;
  dp.nl_on = skin > 0;
  dp.nl_max_cells = max_cells;
  cudaError_t e = cudaSuccess;
  if (dp.nl_on) {
    P.nl_stride = (int)stride;
    P.nl = dalloc<int>((size_t)dp.n_mol * stride, &e);
    P.nl_cnt = dalloc<int>(dp.n_mol, &e);
    P.pbuild = dalloc<float4>(dp.n_pidx, &e);
    P.mcell = dalloc<int>(dp.n_mol, &e);
    P.cell_cnt = dalloc<int>(cells, &e);
    P.cell_start = dalloc<int>(cells, &e);
    P.cell_mol = dalloc<int>(dp.n_mol, &e);
    if (e != cudaSuccess) return set_err(ctx, MCGPU_ERR_NOMEM, "Verlet lists: %s", cudaGetErrorString(e));
  }
  NlCfg* dcfg = dalloc<NlCfg>(nc, &e);
  if (e != cudaSuccess) return set_err(ctx, MCGPU_ERR_NOMEM, "Verlet config: %s", cudaGetErrorString(e));
  e = cudaMemcpyAsync(dcfg, cfg.data(), sizeof(NlCfg) * nc, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    k_nl_config<<<(nc + 127) / 128, 128, 0, st>>>(P, dcfg);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(dcfg);
  if (e != cudaSuccess) return set_err(ctx, MCGPU_ERR_CUDA, "Verlet config: %s", cudaGetErrorString(e));
  return MCGPU_OK;
}

int pool_nl_rebuild(mcgpu_ctx* ctx, DevPool& dp, cudaStream_t st) {
  if (!dp.nl_on) return MCGPU_OK;
  CK(ctx, launch_nl_rebuild(dp.P, dp.mol_chain, dp.n_mol, dp.nl_max_cells, st));
  return MCGPU_OK;
}

// Full system energy of every chain of the pool into dp.esum (device).
int pool_system_energy(mcgpu_ctx* ctx, DevPool& dp, bool f64, cudaStream_t st) {
  const int nw = 4;
  SmemShape sh = shape_for(dp.max_len, nw);
  const int bytes = sh.bytes();
  // split the grid to keep launches moderate
  const int chunk = 1 << 20;
  for (int m0 = 0; m0 < dp.n_mol; m0 += chunk) {
    int n = std::min(chunk, dp.n_mol - m0);
    (void)bytes;
    CK(ctx, launch_mol_pair_sums(f64, n, nw * 32, sh, st, dp.P, dp.mol_chain, m0, dp.emol, dp.pairs));
  }
  k_chain_sums<<<dp.n_chains, 256, 0, st>>>(dp.P, dp.emol, dp.esum);
  CK(ctx, cudaGetLastError());
  return MCGPU_OK;
}

}  // namespace mcgpu

// ---- context ---------------------------------------------------------------------

extern "C" const char* mcgpu_version(void) { return "mcgpu_gb300 0.1 sm_103a"; }

extern "C" int mcgpu_ctx_create(mcgpu_ctx** out, int device) {
  if (!out) return set_err(nullptr, MCGPU_ERR_INVALID, "null output pointer");
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0)
    return set_err(nullptr, MCGPU_ERR_CUDA, "no CUDA device: %s",
                   e != cudaSuccess ? cudaGetErrorString(e) : "0 devices");
  if (device < 0 || device >= n)
    return set_err(nullptr, MCGPU_ERR_INVALID, "device %d out of range [0,%d)", device, n);
  CK(nullptr, cudaSetDevice(device));
  cudaDeviceProp prop;
  CK(nullptr, cudaGetDeviceProperties(&prop, device));
  if (prop.major != 10)
    return set_err(nullptr, MCGPU_ERR_UNSUPPORTED,
                   "device %d is sm_%d%d; this library is built for sm_103a (GB300)", device,
                   prop.major, prop.minor);
  mcgpu_ctx* c = new mcgpu_ctx();
  c->device = device;
  c->sm_count = prop.multiProcessorCount;
  if (cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return set_err(nullptr, MCGPU_ERR_CUDA, "stream creation failed");
  }
  c->stream = c->own;
  if (cudaFuncSetAttribute(k_chain_steps, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           200 * 1024) != cudaSuccess ||
      cudaFuncSetAttribute(k_chain_steps_wide, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           200 * 1024) != cudaSuccess ||
      window_init() != cudaSuccess) {
    cudaStreamDestroy(c->own);
    delete c;
    return set_err(nullptr, MCGPU_ERR_CUDA, "cannot enable large shared memory for the chain kernel");
  }
  *out = c;
  return MCGPU_OK;
}

extern "C" int mcgpu_ctx_destroy(mcgpu_ctx* ctx) {
  if (!ctx) return MCGPU_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->own) cudaStreamDestroy(ctx->own);
  delete ctx;
  return MCGPU_OK;
}

extern "C" int mcgpu_ctx_set_stream(mcgpu_ctx* ctx, void* stream) {
  if (!ctx) return set_err(nullptr, MCGPU_ERR_INVALID, "null context");
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->stream = stream ? (cudaStream_t)stream : ctx->own;
  return MCGPU_OK;
}

extern "C" int mcgpu_last_error(const mcgpu_ctx* ctx, char* buf, size_t len) {
  if (!buf || len == 0) return MCGPU_ERR_INVALID;
  const std::string& s = ctx ? ctx->err : g_err;
  std::snprintf(buf, len, "%s", s.c_str());
  return MCGPU_OK;
}

// ---- box (plain single chain) -------------------------------------------------------

struct mcgpu_box {
  mcgpu_ctx* ctx = nullptr;
  DevPool pool;
  int precision = MCGPU_PREC_FP64;
  int max_grid = 1;
  double* partials = nullptr;
  unsigned* counter = nullptr;
  double* dout = nullptr;
  double* hout = nullptr;  // pinned
  long long* dpairs = nullptr;  // atom pairs the plain energy kernels evaluated
  bool energy_ready = false;
  mcgpu_trace* dtrace = nullptr;
  int trace_cap = 0;
  unsigned* queue = nullptr;
  int* order = nullptr;
  bool chain_state = false;  // pool holds a valid device-resident chain state
  bool rows_stale = false;   // FP64 rows lag the chain state (export before use)
  std::unique_ptr<IntraHost> intra;  // bond / angle rows (flexible molecules)
  bool intra_on = false;             // ENABLE_INTRA for this box
  PlainLoop* dloop = nullptr;        // state of mcgpu_run_plain_device
  int window = 1;                    // steps per window of mcgpu_chain_run (cluster CTAs)
};

// FP64 rows current before a plain entry point reads them.
static int box_rows(mcgpu_box* b) {
  if (!b->rows_stale) return MCGPU_OK;
  int rc = pool_chain_export(b->ctx, b->pool, b->ctx->stream);
  if (rc) return rc;
  b->rows_stale = false;
  return MCGPU_OK;
}

// A plain entry point changed coordinates: the chain state and the running
// energy must be rebuilt before the next device-resident run.
static void box_plain_moved(mcgpu_box* b) {
  b->chain_state = false;
  b->energy_ready = false;
}

// CTAs of a plain energy launch: one per 128 candidates with FP32 pairs, one
// per 32 with FP64 pairs (GB300 runs FP64 at 1/64 of the FP32 rate, so the
// pair work is spread over more SMs).
static int box_grid(const mcgpu_box* b, int n_cand) {
  const int per = b->precision == MCGPU_PREC_FP64 ? 32 : 128;
  int g = (n_cand + per - 1) / per;
  return std::max(1, std::min(g, b->max_grid));
}

// A host-drawn Euler move with its rotation's cosines and sines taken on the
// host by the C library, from the angle in radians formed as the reference
// forms it (SimulationStep.cpp:400-422): the reference's values exactly, and
// no FP64 trigonometry on the device's critical path.
static Proposal host_proposal(const mcgpu_move* mv) {
  Proposal p;
  std::memset(&p, 0, sizeof(p));
  p.vertex = mv->vertex;
  p.mode = MCGPU_ROT_EULER;
  p.dx = mv->dx; p.dy = mv->dy; p.dz = mv->dz;
  p.r0 = mv->rx; p.r1 = mv->ry; p.r2 = mv->rz;
  const double deg[3] = {mv->rx, mv->ry, mv->rz};
  for (int k = 0; k < 3; k++) {
    const double rad = deg[k] * 3.14159265358979 / 180.0;
    p.cs[k] = std::cos(rad);
    p.sn[k] = std::sin(rad);
  }
  p.trig = 1;
  return p;
}

extern "C" int mcgpu_box_upload(mcgpu_ctx* ctx, const mcgpu_box_desc* desc, int precision,
                                mcgpu_box** out) {
  if (!ctx || !desc || !out) return set_err(ctx, MCGPU_ERR_INVALID, "null argument");
  *out = nullptr;
  if (precision != MCGPU_PREC_FP64 && precision != MCGPU_PREC_MIXED)
    return set_err(ctx, MCGPU_ERR_INVALID, "unknown precision %d", precision);
  CK(ctx, cudaSetDevice(ctx->device));
  HostPool hp;
  int rc = append_chain(ctx, hp, desc, 0, 0ull, MCGPU_ROT_EULER);
  if (rc) return rc;
  mcgpu_box* b = new mcgpu_box();
  b->ctx = ctx;
  b->precision = precision;
  rc = upload_pool(ctx, hp, b->pool);
  if (rc) {
    delete b;
    return rc;
  }
  b->max_grid = 4 * ctx->sm_count;
  cudaError_t e = cudaSuccess;
  b->partials = dalloc<double>(2 * (size_t)b->max_grid, &e);
  b->counter = dalloc<unsigned>(2, &e);
  b->dout = dalloc<double>(4, &e);
  b->queue = dalloc<unsigned>(1, &e);
  b->order = dalloc<int>(1, &e);
  if (e == cudaSuccess) e = cudaMallocHost((void**)&b->hout, 4 * sizeof(double));
  if (e == cudaSuccess) e = cudaMemsetAsync(b->counter, 0, 2 * sizeof(unsigned), ctx->stream);
  if (e == cudaSuccess) b->dpairs = dalloc<long long>(1, &e);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->dpairs, 0, sizeof(long long), ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->order, 0, sizeof(int), ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    mcgpu_box_destroy(b);
    return set_err(ctx, MCGPU_ERR_NOMEM, "box scratch allocation failed: %s", cudaGetErrorString(e));
  }
  *out = b;
  return MCGPU_OK;
}

extern "C" int mcgpu_box_destroy(mcgpu_box* b) {
  if (!b) return MCGPU_OK;
  cudaSetDevice(b->ctx->device);
  cudaStreamSynchronize(b->ctx->stream);
  b->pool.release();
  if (b->partials) cudaFree(b->partials);
  if (b->counter) cudaFree(b->counter);
  if (b->dout) cudaFree(b->dout);
  if (b->hout) cudaFreeHost(b->hout);
  if (b->dpairs) cudaFree(b->dpairs);
  if (b->dloop) cudaFree(b->dloop);
  if (b->dtrace) cudaFree(b->dtrace);
  if (b->queue) cudaFree(b->queue);
  if (b->order) cudaFree(b->order);
  delete b;
  return MCGPU_OK;
}

extern "C" int mcgpu_box_download(mcgpu_box* b, double* x, double* y, double* z, double* size) {
  if (!b || !x || !y || !z) return set_err(b ? b->ctx : nullptr, MCGPU_ERR_INVALID, "null argument");
  mcgpu_ctx* ctx = b->ctx;
  int rc = box_rows(b);
  if (rc) return rc;
  const size_t n = (size_t)b->pool.n_atom;
  CK(ctx, cudaMemcpyAsync(x, b->pool.P.x, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaMemcpyAsync(y, b->pool.P.y, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaMemcpyAsync(z, b->pool.P.z, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  if (size)
    for (int k = 0; k < 3; k++) size[k] = b->pool.hdr[0].L[k];
  return MCGPU_OK;
}

extern "C" int mcgpu_mol_energy(mcgpu_box* b, int curr, int start, double* out) {
  if (!b || !out) return set_err(b ? b->ctx : nullptr, MCGPU_ERR_INVALID, "null argument");
  mcgpu_ctx* ctx = b->ctx;
  const int n = b->pool.n_mol;
  if (curr < 0 || curr >= n) return set_err(ctx, MCGPU_ERR_INVALID, "molecule %d out of [0,%d)", curr, n);
  if (start < 0 || start > n) return set_err(ctx, MCGPU_ERR_INVALID, "start %d out of [0,%d]", start, n);
  if (start == n) {
    *out = 0.0;
    return b->intra_on ? mcgpu_intra_energy(b, curr, out) : MCGPU_OK;
  }
  int rc = box_rows(b);
  if (rc) return rc;
  const int nw = 4;
  SmemShape sh = shape_for(b->pool.max_len, nw);
  const int grid = box_grid(b, n - start);
  CK(ctx, launch_mol_energy(b->precision == MCGPU_PREC_FP64, grid, nw * 32, sh, ctx->stream,
                            b->pool.P, 0, curr, start, b->partials, b->counter, b->dout,
                            b->dpairs));
  if (b->intra_on) {
    // SimulationStep::calcMoleculeEnergy with ENABLE_INTRA (SimulationStep.cpp:15-18)
    CK(ctx, launch_intra_energy(b->pool.P, b->intra->R, 0, curr, b->dout + 1, ctx->stream));
    CK(ctx, cudaMemcpyAsync(b->hout, b->dout, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                            ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    *out = b->hout[0] + b->hout[1];
    return MCGPU_OK;
  }
  CK(ctx, cudaMemcpyAsync(b->hout, b->dout, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  *out = b->hout[0];
  return MCGPU_OK;
}

static int check_move(mcgpu_box* b, int mol, const mcgpu_move* mv) {
  mcgpu_ctx* ctx = b->ctx;
  if (!mv) return set_err(ctx, MCGPU_ERR_INVALID, "null move");
  if (mol < 0 || mol >= b->pool.n_mol)
    return set_err(ctx, MCGPU_ERR_INVALID, "molecule %d out of [0,%d)", mol, b->pool.n_mol);
  const int len = b->pool.mlen[mol] & 255;
  if (mv->vertex < 0 || mv->vertex >= len)
    return set_err(ctx, MCGPU_ERR_INVALID, "vertex %d out of [0,%d) for molecule %d", mv->vertex,
                   len, mol);
  if (!std::isfinite(mv->dx) || !std::isfinite(mv->dy) || !std::isfinite(mv->dz) ||
      !std::isfinite(mv->rx) || !std::isfinite(mv->ry) || !std::isfinite(mv->rz))
    return set_err(ctx, MCGPU_ERR_INVALID, "non-finite move");
  return MCGPU_OK;
}

extern "C" int mcgpu_change_molecule(mcgpu_box* b, int mol, const mcgpu_move* mv) {
  if (!b) return set_err(nullptr, MCGPU_ERR_INVALID, "null box");
  int rc = check_move(b, mol, mv);
  if (rc) return rc;
  rc = box_rows(b);
  if (rc) return rc;
  box_plain_moved(b);
  mcgpu_ctx* ctx = b->ctx;
  SmemShape sh = shape_for(b->pool.max_len, 1);
  k_change_molecule<<<1, 32, sh.bytes(), ctx->stream>>>(b->pool.P, 0, mol, host_proposal(mv), sh);
  CK(ctx, cudaGetLastError());
  // SimCalcs::changeMolecule with ENABLE_INTRA (SimulationStep.cpp:424-428)
  if (b->intra_on) return mcgpu_intramolecular_move(b, mol);
  return MCGPU_OK;
}

extern "C" int mcgpu_rollback(mcgpu_box* b, int mol) {
  if (!b) return set_err(nullptr, MCGPU_ERR_INVALID, "null box");
  mcgpu_ctx* ctx = b->ctx;
  if (mol < 0 || mol >= b->pool.n_mol)
    return set_err(ctx, MCGPU_ERR_INVALID, "molecule %d out of [0,%d)", mol, b->pool.n_mol);
  int rc = box_rows(b);
  if (rc) return rc;
  box_plain_moved(b);
  if (b->intra_on) {
    // SimCalcs::rollback's ENABLE_INTRA branch (SimulationStep.cpp:745-748)
    CK(ctx, launch_intra_rollback(b->pool.P, b->intra->R, 0, mol, ctx->stream));
    return MCGPU_OK;
  }
  k_rollback<<<1, 32, 0, ctx->stream>>>(b->pool.P, 0, mol);
  CK(ctx, cudaGetLastError());
  return MCGPU_OK;
}

extern "C" int mcgpu_move_energies(mcgpu_box* b, int mol, const mcgpu_move* mv, double* e_old,
                                   double* e_new) {
  if (!b || !e_old || !e_new) return set_err(b ? b->ctx : nullptr, MCGPU_ERR_INVALID, "null argument");
  if (b->intra_on)
    return set_err(b->ctx, MCGPU_ERR_UNSUPPORTED,
                   "mcgpu_move_energies moves rigid molecules; with intramolecular moves on use "
                   "mcgpu_mol_energy and mcgpu_change_molecule");
  int rc = check_move(b, mol, mv);
  if (rc) return rc;
  rc = box_rows(b);
  if (rc) return rc;
  box_plain_moved(b);
  mcgpu_ctx* ctx = b->ctx;
  const int nw = 4;
  SmemShape sh = shape_for(b->pool.max_len, nw);
  const int grid = box_grid(b, b->pool.n_mol);
  CK(ctx, launch_move_energies(b->precision == MCGPU_PREC_FP64, grid, nw * 32, sh, ctx->stream,
                               b->pool.P, 0, mol, host_proposal(mv), b->partials, b->counter,
                               b->dout, b->dpairs));
  CK(ctx, cudaMemcpyAsync(b->hout, b->dout, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  *e_old = b->hout[0];
  *e_new = b->hout[1];
  return MCGPU_OK;
}

extern "C" int mcgpu_system_energy(mcgpu_box* b, double* out) {
  if (!b || !out) return set_err(b ? b->ctx : nullptr, MCGPU_ERR_INVALID, "null argument");
  mcgpu_ctx* ctx = b->ctx;
  int rc = box_rows(b);
  if (rc) return rc;
  if (b->intra_on) {
    // calcSystemEnergy with ENABLE_INTRA: molecule m adds E(m, j > m) and its
    // intramolecular energy (SimulationStep.cpp:40-71 over :15-18)
    DevPool& dp = b->pool;
    const int nw = 4;
    SmemShape sh = shape_for(dp.max_len, nw);
    const int chunk = 1 << 20;
    for (int m0 = 0; m0 < dp.n_mol; m0 += chunk)
      CK(ctx, launch_mol_pair_sums(b->precision == MCGPU_PREC_FP64,
                                   std::min(chunk, dp.n_mol - m0), nw * 32, sh, ctx->stream,
                                   dp.P, dp.mol_chain, m0, dp.emol, dp.pairs));
    CK(ctx, launch_intra_add(dp.P, b->intra->R, dp.n_mol, dp.emol, ctx->stream));
    k_chain_sums<<<dp.n_chains, 256, 0, ctx->stream>>>(dp.P, dp.emol, dp.esum);
    CK(ctx, cudaGetLastError());
  } else {
    rc = pool_system_energy(ctx, b->pool, b->precision == MCGPU_PREC_FP64, ctx->stream);
    if (rc) return rc;
  }
  CK(ctx, cudaMemcpyAsync(b->hout, b->pool.esum, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  *out = b->hout[0];
  return MCGPU_OK;
}

// ---- the reference's NVT loop over the contract, in C++ -------------------

namespace {
// randomReal of the reference (MathLibrary.cpp:31-33) over the C library's
// rand(), seeded with srand().
double random_real(double start, double end) {
  return (end - start) * ((double)std::rand() / RAND_MAX) + start;
}
}  // namespace

static int run_plain_intra(mcgpu_box* b, int n_steps, mcgpu_plain_stats* out, double& e);

// The rigid loop: the contract calls one after another (or the fused
// energy-move-energy call), as a GpuBruteForceStep sees them.
static int run_plain_rigid(mcgpu_box* b, int n_steps, int fused, mcgpu_plain_stats* out,
                           double& e) {
  const ChainHdr& h = b->pool.hdr[0];
  const int n = b->pool.n_mol;
  const double kT = h.kT, max_t = h.max_t, max_r = h.max_r;
  for (int step = 0; step < n_steps; step++) {
    // chooseMolecule (SimulationStep.cpp:25-27); rand() == RAND_MAX gives n,
    // clamped to n - 1 (the reference would read past its rows)
    const int mol = std::min((int)random_real(0, n), n - 1);
    // the seven draws of intermolecularMove (SimulationStep.cpp:527-535)
    const int len = b->pool.mlen[mol] & 255;
    mcgpu_move mv;
    std::memset(&mv, 0, sizeof(mv));
    mv.vertex = std::min((int)random_real(0, len), len - 1);
    mv.dx = random_real(-max_t, max_t);
    mv.dy = random_real(-max_t, max_t);
    mv.dz = random_real(-max_t, max_t);
    mv.rx = random_real(-max_r, max_r);
    mv.ry = random_real(-max_r, max_r);
    mv.rz = random_real(-max_r, max_r);
    double e_old = 0.0, e_new = 0.0;
    int rc;
    if (fused) {
      rc = mcgpu_move_energies(b, mol, &mv, &e_old, &e_new);
    } else {
      rc = mcgpu_mol_energy(b, mol, 0, &e_old);
      if (!rc) rc = mcgpu_change_molecule(b, mol, &mv);
      if (!rc) rc = mcgpu_mol_energy(b, mol, 0, &e_new);
    }
    if (rc) return rc;
    // acceptMove (SimulationStep.cpp:794-803)
    const double de = e_new - e_old;
    const bool ok = de < 0 || std::exp(-de / kT) >= random_real(0.0, 1.0);
    if (ok) {
      e += de;
      out->accepted++;
    } else {
      out->rejected++;
      rc = mcgpu_rollback(b, mol);
      if (rc) return rc;
    }
  }
  return MCGPU_OK;
}

extern "C" int mcgpu_run_plain(mcgpu_box* b, unsigned int seed, int n_steps, int fused,
                               mcgpu_plain_stats* out) {
  if (!b || !out) return set_err(b ? b->ctx : nullptr, MCGPU_ERR_INVALID, "null argument");
  mcgpu_ctx* ctx = b->ctx;
  if (n_steps < 0) return set_err(ctx, MCGPU_ERR_INVALID, "negative step count");
  std::memset(out, 0, sizeof(*out));
  CK(ctx, cudaMemsetAsync(b->dpairs, 0, sizeof(long long), ctx->stream));
  double e = 0.0;
  int rc = mcgpu_system_energy(b, &e);
  if (rc) return rc;
  out->energy0 = e;
  std::srand(seed);
  rc = b->intra_on ? run_plain_intra(b, n_steps, out, e)
                   : run_plain_rigid(b, n_steps, fused, out, e);
  if (rc) return rc;
  long long np = 0;
  CK(ctx, cudaMemcpyAsync(&np, b->dpairs, sizeof(long long), cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  out->energy = e;
  out->pairs = np;
  return MCGPU_OK;
}

// The same loop on the device: one CTA per box runs the steps with the
// restated C-library generator, launches of kDeviceLoopSteps steps.
static constexpr int kDeviceLoopSteps = 4096;

extern "C" int mcgpu_boxes_run_plain_device(mcgpu_box* const* boxes, int n_boxes,
                                            const unsigned int* seeds, int n_steps,
                                            mcgpu_plain_stats* out) {
  if (!boxes || !seeds || !out || n_boxes < 1)
    return set_err(nullptr, MCGPU_ERR_INVALID, "null argument or no boxes");
  mcgpu_box* b0 = boxes[0];
  if (!b0) return set_err(nullptr, MCGPU_ERR_INVALID, "null box");
  mcgpu_ctx* ctx = b0->ctx;
  if (n_steps < 0) return set_err(ctx, MCGPU_ERR_INVALID, "negative step count");
  int max_len = 0;
  for (int i = 0; i < n_boxes; i++) {
    mcgpu_box* b = boxes[i];
    if (!b) return set_err(ctx, MCGPU_ERR_INVALID, "null box %d", i);
    if (b->ctx != ctx) return set_err(ctx, MCGPU_ERR_INVALID, "box %d: another context", i);
    if (b->precision != b0->precision)
      return set_err(ctx, MCGPU_ERR_INVALID, "box %d: another pair precision", i);
    for (int j = 0; j < i; j++)
      if (boxes[j] == b) return set_err(ctx, MCGPU_ERR_INVALID, "box %d given twice", i);
    if (b->intra_on && b->intra->max_intra_moves > kLoopSel)
      return set_err(ctx, MCGPU_ERR_UNSUPPORTED, "box %d: max_intra_moves %d above %d", i,
                     b->intra->max_intra_moves, kLoopSel);
    max_len = std::max(max_len, b->pool.max_len);
  }
  std::vector<LoopTask> tasks(n_boxes);
  std::vector<PlainLoop> loops(n_boxes);
  for (int i = 0; i < n_boxes; i++) {
    mcgpu_box* b = boxes[i];
    mcgpu_plain_stats& o = out[i];
    std::memset(&o, 0, sizeof(o));
    double e = 0.0;
    int rc = mcgpu_system_energy(b, &e);
    if (rc) return rc;
    o.energy0 = e;
    if (!b->dloop) CK(ctx, cudaMalloc((void**)&b->dloop, sizeof(PlainLoop)));
    PlainLoop& L = loops[i];
    std::memset(&L, 0, sizeof(L));
    crand_seed(L.rng, seeds[i]);
    L.energy = e;
    LoopTask& T = tasks[i];
    std::memset(&T, 0, sizeof(T));
    T.P = b->pool.P;
    T.L = b->dloop;
    T.intra = b->intra_on ? 1 : 0;
    if (b->intra_on) {
      IntraHost& I = *b->intra;
      T.R = I.R;
      L.step = I.step;
      L.max_bond_delta = I.max_bond_delta;
      L.max_angle_delta = I.max_angle_delta;
      L.bond_moves = I.bond_moves;
      L.bond_accepted = I.bond_accepted;
      L.angle_moves = I.angle_moves;
      L.angle_accepted = I.angle_accepted;
      L.max_intra_moves = I.max_intra_moves;
    }
    CK(ctx, cudaMemcpyAsync(b->dloop, &L, sizeof(L), cudaMemcpyHostToDevice, ctx->stream));
  }
  LoopTask* dt = nullptr;
  CK(ctx, cudaMalloc((void**)&dt, sizeof(LoopTask) * n_boxes));
  cudaError_t e = cudaMemcpyAsync(dt, tasks.data(), sizeof(LoopTask) * n_boxes,
                                  cudaMemcpyHostToDevice, ctx->stream);
  SmemShape sh = shape_for(max_len, 8);
  for (int done = 0; e == cudaSuccess && done < n_steps; done += kDeviceLoopSteps)
    e = launch_plain_steps(b0->precision == MCGPU_PREC_FP64, dt, n_boxes,
                           std::min(kDeviceLoopSteps, n_steps - done), sh, ctx->stream);
  for (int i = 0; e == cudaSuccess && i < n_boxes; i++)
    e = cudaMemcpyAsync(&loops[i], boxes[i]->dloop, sizeof(PlainLoop), cudaMemcpyDeviceToHost,
                        ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(dt);
  if (e != cudaSuccess)
    return set_err(ctx, MCGPU_ERR_CUDA, "device loop failed: %s", cudaGetErrorString(e));
  for (int i = 0; i < n_boxes; i++) {
    mcgpu_box* b = boxes[i];
    const PlainLoop& L = loops[i];
    box_plain_moved(b);
    if (L.error)
      return set_err(ctx, MCGPU_ERR_DEVICE, "box %d: an intramolecular stage's index draws did "
                     "not fill its set (device loop stopped after %lld steps)", i,
                     L.accepted + L.rejected);
    if (b->intra_on) {
      IntraHost& I = *b->intra;
      I.step = L.step;
      I.max_bond_delta = L.max_bond_delta;
      I.max_angle_delta = L.max_angle_delta;
      I.bond_moves = L.bond_moves;
      I.bond_accepted = L.bond_accepted;
      I.angle_moves = L.angle_moves;
      I.angle_accepted = L.angle_accepted;
    }
    out[i].energy = L.energy;
    out[i].accepted = L.accepted;
    out[i].rejected = L.rejected;
    out[i].pairs = L.pairs;
  }
  return MCGPU_OK;
}

extern "C" int mcgpu_run_plain_device(mcgpu_box* b, unsigned int seed, int n_steps,
                                      mcgpu_plain_stats* out) {
  if (!b || !out) return set_err(b ? b->ctx : nullptr, MCGPU_ERR_INVALID, "null argument");
  return mcgpu_boxes_run_plain_device(&b, 1, &seed, n_steps, out);
}

extern "C" int mcgpu_rand_stream(unsigned int seed, int n, int32_t* out) {
  if (n < 0 || (n && !out)) return set_err(nullptr, MCGPU_ERR_INVALID, "bad argument");
  CRand g;
  crand_seed(g, seed);
  for (int k = 0; k < n; k++) out[k] = crand_next(g);
  return MCGPU_OK;
}

// ---- flexible molecules ----------------------------------------------------------

extern "C" int mcgpu_box_set_topology(mcgpu_box* b, const mcgpu_topology_desc* t) {
  if (!b) return set_err(nullptr, MCGPU_ERR_INVALID, "null box");
  mcgpu_ctx* ctx = b->ctx;
  int rc = box_rows(b);
  if (rc) return rc;
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  const DevPool& dp = b->pool;
  std::vector<int> len(dp.n_mol);
  for (int m = 0; m < dp.n_mol; m++) len[m] = dp.mlen[m] & 255;  // atoms | active << 8
  std::unique_ptr<IntraHost> I;
  rc = intra_upload(ctx, dp.n_mol, dp.n_atom, dp.mstart.data(), len.data(), t, &I);
  if (rc) return rc;
  b->intra = std::move(I);
  box_plain_moved(b);
  return MCGPU_OK;
}

extern "C" int mcgpu_box_set_intra(mcgpu_box* b, int enable) {
  if (!b) return set_err(nullptr, MCGPU_ERR_INVALID, "null box");
  if (enable && !b->intra)
    return set_err(b->ctx, MCGPU_ERR_INVALID, "intramolecular moves need a topology");
  b->intra_on = enable != 0;
  box_plain_moved(b);
  return MCGPU_OK;
}

static int intra_checks(mcgpu_box* b, int mol) {
  if (!b) return set_err(nullptr, MCGPU_ERR_INVALID, "null box");
  if (!b->intra) return set_err(b->ctx, MCGPU_ERR_INVALID, "the box has no topology");
  if (mol < 0 || mol >= b->pool.n_mol)
    return set_err(b->ctx, MCGPU_ERR_INVALID, "molecule %d out of [0,%d)", mol, b->pool.n_mol);
  return box_rows(b);
}

extern "C" int mcgpu_intra_energy(mcgpu_box* b, int mol, double* out) {
  int rc = intra_checks(b, mol);
  if (rc) return rc;
  if (!out) return set_err(b->ctx, MCGPU_ERR_INVALID, "null argument");
  mcgpu_ctx* ctx = b->ctx;
  IntraHost& I = *b->intra;
  CK(ctx, launch_intra_energy(b->pool.P, I.R, 0, mol, I.dout, ctx->stream));
  CK(ctx, cudaMemcpyAsync(I.hout, I.dout, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  *out = I.hout[0];
  return MCGPU_OK;
}

// SimCalcs::expandAngle's constant (SimulationStep.cpp:181): its digits
// differ from pi's after the seventh; kept, since the moved coordinates
// depend on it.
static const double kIntraDeg2Rad = 3.14159256358979323846264 / 180.0;

// The cosines and sines of an expansion's two group angles, by the C
// library, from the angles formed as the reference forms them.
static void angle_trig(IntraOps& ops, int k, double deg) {
  const double t1 = deg * -kIntraDeg2Rad, t2 = deg * kIntraDeg2Rad;
  ops.c1[k] = std::cos(t1);
  ops.s1[k] = std::sin(t1);
  ops.c2[k] = std::cos(t2);
  ops.s2[k] = std::sin(t2);
}

// Launches ops (kind 0 bonds, 1 angles) of molecule mol in launches of
// kIntraOps, the first with `first_flags`, the last with the energy after
// (into the topology's device out[0..1]); no wait.
static int intra_launch_ops(mcgpu_box* b, int mol, int kind, const std::vector<int>& idx,
                            const std::vector<double>& amt, int first_flags, bool energy_after) {
  mcgpu_ctx* ctx = b->ctx;
  IntraHost& I = *b->intra;
  const int n = (int)idx.size();
  int done = 0;
  do {
    IntraOps ops;
    std::memset(&ops, 0, sizeof(ops));
    ops.mol = mol;
    ops.kind = kind;
    ops.n = std::min(kIntraOps, n - done);
    for (int k = 0; k < ops.n; k++) {
      ops.idx[k] = idx[done + k];
      ops.amt[k] = amt[done + k];
      if (kind == 1) angle_trig(ops, k, amt[done + k]);
    }
    ops.flags = done == 0 ? first_flags : 0;
    if (done + ops.n >= n && energy_after) ops.flags |= kIntraEnergyAfter;
    CK(ctx, launch_intra_ops(b->pool.P, I.R, 0, ops, I.dout, ctx->stream));
    done += ops.n;
  } while (done < n);
  box_plain_moved(b);
  return MCGPU_OK;
}

// intra_launch_ops, then the stage's energies in the topology's host out[0..1].
static int intra_run_ops(mcgpu_box* b, int mol, int kind, const std::vector<int>& idx,
                         const std::vector<double>& amt, int first_flags, bool energy_after) {
  int rc = intra_launch_ops(b, mol, kind, idx, amt, first_flags, energy_after);
  if (rc) return rc;
  if (first_flags & kIntraEnergyBefore || energy_after) {
    mcgpu_ctx* ctx = b->ctx;
    IntraHost& I = *b->intra;
    CK(ctx, cudaMemcpyAsync(I.hout, I.dout, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                            ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
  }
  return MCGPU_OK;
}

extern "C" int mcgpu_stretch_bond(mcgpu_box* b, int mol, int bond, double dist) {
  int rc = intra_checks(b, mol);
  if (rc) return rc;
  if (bond < 0 || bond >= b->intra->bcount[mol])
    return set_err(b->ctx, MCGPU_ERR_INVALID, "bond %d out of [0,%d) for molecule %d", bond,
                   b->intra->bcount[mol], mol);
  return intra_run_ops(b, mol, 0, {bond}, {dist}, 0, false);
}

extern "C" int mcgpu_expand_angle(mcgpu_box* b, int mol, int angle, double deg) {
  int rc = intra_checks(b, mol);
  if (rc) return rc;
  if (angle < 0 || angle >= b->intra->acount[mol])
    return set_err(b->ctx, MCGPU_ERR_INVALID, "angle %d out of [0,%d) for molecule %d", angle,
                   b->intra->acount[mol], mol);
  return intra_run_ops(b, mol, 1, {angle}, {deg}, 0, false);
}

extern "C" int mcgpu_save_intra(mcgpu_box* b, int mol) {
  int rc = intra_checks(b, mol);
  if (rc) return rc;
  return intra_run_ops(b, mol, 0, {}, {}, kIntraSave, false);
}

// The distinct indexes std::set collects from (int)randomReal(0, count)
// draws until it holds `want` (SimulationStep.cpp:599-601, 631-633), in the
// set's ascending order; a draw of count (rand() == RAND_MAX) is taken as
// count - 1 (the reference would index past the molecule's rows).
static void intra_draw_set(int want, int count, std::vector<int>& out) {
  out.clear();
  while ((int)out.size() < want) {
    int v = std::min((int)random_real(0, count), count - 1);
    auto it = std::lower_bound(out.begin(), out.end(), v);
    if (it != out.end() && *it == v) continue;
    out.insert(it, v);
  }
}

// The draws of one stage of SimCalcs::intramolecularMove (kind 0: bonds,
// :589-609; kind 1: angles, :621-640) with the entry width `delta`: how many
// (2 move types, ENABLE_BOND + ENABLE_ANGLE), which, and an amount for each
// drawn whether or not the entry is variable; idx / amt keep the variable
// ones.  Returns the count the move counters take.
static int intra_draw_stage(IntraHost& I, int mol, int kind, double delta,
                            std::vector<int>& idx, std::vector<double>& amt) {
  const double intra_scale = 0.25 + (0.75 / (double)2);
  const int count = kind == 0 ? I.bcount[mol] : I.acount[mol];
  const int start = kind == 0 ? I.bstart[mol] : I.astart[mol];
  const std::vector<int>& var = kind == 0 ? I.bvar : I.avar;
  int n = count;
  if (n > 3) n = std::min((int)random_real(2, count), I.max_intra_moves);
  const double scale = 0.25 + (0.75 / (double)n) * intra_scale;
  std::vector<int> set;
  intra_draw_set(n, count, set);
  idx.clear();
  amt.clear();
  for (int k : set) {
    const double d = scale * random_real(-delta, delta);
    if (var[start + k]) {
      idx.push_back(k);
      amt.push_back(d);
    }
  }
  return n;
}

// acceptMove (SimulationStep.cpp:794-803): a decrease is accepted without a
// draw, otherwise exp(-dE/kT) against a uniform from rand().
static bool host_accept(double de, double kT) {
  return de < 0 || std::exp(-(de) / kT) >= random_real(0.0, 1.0);
}

// The width tuning at the end of SimCalcs::intramolecularMove (:656-674):
// TARGET_RATIO 0.4, RATIO_MARGIN 1e-4; the angle test reads the entry width,
// as the reference's does.
static void intra_tune(IntraHost& I, double angle_delta) {
  if (I.step == 0 || (I.step % 1000) != 0) return;
  const double bond_ratio = (double)I.bond_accepted / I.bond_moves;
  const double angle_ratio = (double)I.angle_accepted / I.angle_moves;
  double diff = bond_ratio - 0.4;
  if (std::fabs(diff) > 0.0001) I.max_bond_delta += I.max_bond_delta * diff;
  diff = angle_ratio - 0.4;
  if (std::fabs(angle_delta) > 0.0001) I.max_angle_delta += I.max_angle_delta * diff;
  I.bond_accepted = I.bond_moves = 0;
  I.angle_accepted = I.angle_moves = 0;
}

extern "C" int mcgpu_intramolecular_move(mcgpu_box* b, int mol) {
  int rc = intra_checks(b, mol);
  if (rc) return rc;
  IntraHost& I = *b->intra;
  const double kT = b->pool.hdr[0].kT;
  const double bond_delta = I.max_bond_delta, angle_delta = I.max_angle_delta;
  std::vector<int> idx;
  std::vector<double> amt;
  bool saved = false;
  double cur_e = 0.0;
  if (I.flex_bonds) {
    const int n = intra_draw_stage(I, mol, 0, bond_delta, idx, amt);
    I.bond_moves += n;
    rc = intra_run_ops(b, mol, 0, idx, amt, kIntraSave | kIntraEnergyBefore, true);
    if (rc) return rc;
    saved = true;
    if (host_accept(I.hout[1] - I.hout[0], kT)) I.bond_accepted += n;
    cur_e = I.hout[1];
  }
  if (I.flex_angles) {
    const int n = intra_draw_stage(I, mol, 1, angle_delta, idx, amt);
    I.angle_moves += n;
    rc = intra_run_ops(b, mol, 1, idx, amt, saved ? 0 : (kIntraSave | kIntraEnergyBefore), true);
    if (rc) return rc;
    if (!saved) cur_e = I.hout[0];
    if (host_accept(I.hout[1] - cur_e, kT)) I.angle_accepted += n;
  }
  intra_tune(I, angle_delta);
  return MCGPU_OK;
}

// mcgpu_run_plain's loop with intramolecular moves: the calls and draws of
// the reference's loop with ENABLE_INTRA, launched so that each step waits
// on the device twice.  Draws that do not depend on an energy are taken
// ahead: molecule, the rigid move and the bond stage's draws go before the
// first wait, with the old energy, the rigid move and the bond stage
// launched behind them; the bond test's uniform (when drawn) and the angle
// stage's draws go before the second wait, behind which run the angle stage
// and the new energy.  The draw order and every value are those of the
// one-call-at-a-time sequence.
static int run_plain_intra(mcgpu_box* b, int n_steps, mcgpu_plain_stats* out, double& e) {
  mcgpu_ctx* ctx = b->ctx;
  IntraHost& I = *b->intra;
  const ChainHdr& h = b->pool.hdr[0];
  const int n = b->pool.n_mol;
  const double kT = h.kT, max_t = h.max_t, max_r = h.max_r;
  const bool f64 = b->precision == MCGPU_PREC_FP64;
  const int nw = 4;
  SmemShape sh = shape_for(b->pool.max_len, nw);
  SmemShape sh1 = shape_for(b->pool.max_len, 1);
  const int grid = box_grid(b, n);
  const long long step0 = I.step;
  std::vector<int> idx;
  std::vector<double> amt;
  double* hv = b->hout;   // [0] inter, [1] intra (host copies), [2..3] stage energies
  for (int step = 0; step < n_steps; step++) {
    I.step = step0 + step;
    const int mol = std::min((int)random_real(0, n), n - 1);
    const int len = b->pool.mlen[mol] & 255;
    mcgpu_move mv;
    std::memset(&mv, 0, sizeof(mv));
    mv.vertex = std::min((int)random_real(0, len), len - 1);
    mv.dx = random_real(-max_t, max_t);
    mv.dy = random_real(-max_t, max_t);
    mv.dz = random_real(-max_t, max_t);
    mv.rx = random_real(-max_r, max_r);
    mv.ry = random_real(-max_r, max_r);
    mv.rz = random_real(-max_r, max_r);
    const double bond_delta = I.max_bond_delta, angle_delta = I.max_angle_delta;
    // old energy (inter + intra), the rigid move, the bond stage
    CK(ctx, launch_mol_energy(f64, grid, nw * 32, sh, ctx->stream, b->pool.P, 0, mol, 0,
                              b->partials, b->counter, b->dout, b->dpairs));
    CK(ctx, launch_intra_energy(b->pool.P, I.R, 0, mol, b->dout + 1, ctx->stream));
    k_change_molecule<<<1, 32, sh1.bytes(), ctx->stream>>>(b->pool.P, 0, mol,
                                                           host_proposal(&mv), sh1);
    CK(ctx, cudaGetLastError());
    box_plain_moved(b);
    int nb = 0;
    if (I.flex_bonds) {
      nb = intra_draw_stage(I, mol, 0, bond_delta, idx, amt);
      I.bond_moves += nb;
      int rc = intra_launch_ops(b, mol, 0, idx, amt, kIntraSave | kIntraEnergyBefore, true);
      if (rc) return rc;
    }
    CK(ctx, cudaMemcpyAsync(hv, b->dout, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                            ctx->stream));
    if (I.flex_bonds)
      CK(ctx, cudaMemcpyAsync(I.hout, I.dout, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                              ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    const double e_old = hv[0] + hv[1];
    double cur_e = 0.0;
    if (I.flex_bonds) {
      if (host_accept(I.hout[1] - I.hout[0], kT)) I.bond_accepted += nb;
      cur_e = I.hout[1];
    }
    // the angle stage and the new energy
    int na = 0;
    if (I.flex_angles) {
      na = intra_draw_stage(I, mol, 1, angle_delta, idx, amt);
      I.angle_moves += na;
      int rc = intra_launch_ops(b, mol, 1, idx, amt,
                                I.flex_bonds ? 0 : (kIntraSave | kIntraEnergyBefore), true);
      if (rc) return rc;
    }
    CK(ctx, launch_mol_energy(f64, grid, nw * 32, sh, ctx->stream, b->pool.P, 0, mol, 0,
                              b->partials, b->counter, b->dout, b->dpairs));
    CK(ctx, launch_intra_energy(b->pool.P, I.R, 0, mol, b->dout + 1, ctx->stream));
    CK(ctx, cudaMemcpyAsync(hv, b->dout, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                            ctx->stream));
    if (I.flex_angles)
      CK(ctx, cudaMemcpyAsync(I.hout, I.dout, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                              ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    if (I.flex_angles) {
      if (!I.flex_bonds) cur_e = I.hout[0];
      if (host_accept(I.hout[1] - cur_e, kT)) I.angle_accepted += na;
    }
    intra_tune(I, angle_delta);
    const double e_new = hv[0] + hv[1];
    const double de = e_new - e_old;
    if (host_accept(de, kT)) {
      e += de;
      out->accepted++;
    } else {
      out->rejected++;
      CK(ctx, launch_intra_rollback(b->pool.P, I.R, 0, mol, ctx->stream));
    }
  }
  I.step = step0 + n_steps;
  return MCGPU_OK;
}

extern "C" int mcgpu_intra_set_step(mcgpu_box* b, int64_t step) {
  if (!b) return set_err(nullptr, MCGPU_ERR_INVALID, "null box");
  if (!b->intra) return set_err(b->ctx, MCGPU_ERR_INVALID, "the box has no topology");
  b->intra->step = step;
  return MCGPU_OK;
}

extern "C" int mcgpu_intra_get(mcgpu_box* b, double* bond_len, double* angle_size,
                               mcgpu_intra_state* state) {
  if (!b) return set_err(nullptr, MCGPU_ERR_INVALID, "null box");
  if (!b->intra) return set_err(b->ctx, MCGPU_ERR_INVALID, "the box has no topology");
  mcgpu_ctx* ctx = b->ctx;
  IntraHost& I = *b->intra;
  if (bond_len && I.n_bond)
    CK(ctx, cudaMemcpyAsync(bond_len, I.R.b_len, sizeof(double) * I.n_bond,
                            cudaMemcpyDeviceToHost, ctx->stream));
  if (angle_size && I.n_angle)
    CK(ctx, cudaMemcpyAsync(angle_size, I.R.a_size, sizeof(double) * I.n_angle,
                            cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  if (state) {
    state->max_bond_delta = I.max_bond_delta;
    state->max_angle_delta = I.max_angle_delta;
    state->step_num = I.step;
    state->bond_moves = I.bond_moves;
    state->bond_accepted = I.bond_accepted;
    state->angle_moves = I.angle_moves;
    state->angle_accepted = I.angle_accepted;
  }
  return MCGPU_OK;
}

extern "C" int mcgpu_chain_run(mcgpu_box* b, uint64_t seed, uint32_t chain_id, int n_steps,
                               int rotation, mcgpu_chain_stats* stats, mcgpu_trace* trace) {
  if (!b) return set_err(nullptr, MCGPU_ERR_INVALID, "null box");
  mcgpu_ctx* ctx = b->ctx;
  if (n_steps < 0) return set_err(ctx, MCGPU_ERR_INVALID, "negative step count");
  if (rotation != MCGPU_ROT_EULER && rotation != MCGPU_ROT_AXIS)
    return set_err(ctx, MCGPU_ERR_INVALID, "unknown rotation form %d", rotation);
  if (b->intra_on)
    return set_err(ctx, MCGPU_ERR_UNSUPPORTED,
                   "the device-resident chain moves rigid molecules; intramolecular moves run "
                   "on the plain path");
  cudaStream_t st = ctx->stream;
  DevPool& dp = b->pool;
  ChainHdr* dh = dp.P.hdr;
  // key, counter chain id and rotation form of this run
  CK(ctx, cudaMemcpyAsync(&dh->seed, &seed, 8, cudaMemcpyHostToDevice, st));
  int cid = (int)chain_id;
  CK(ctx, cudaMemcpyAsync(&dh->chain_id, &cid, 4, cudaMemcpyHostToDevice, st));
  CK(ctx, cudaMemcpyAsync(&dh->rot_mode, &rotation, 4, cudaMemcpyHostToDevice, st));
  if (!b->chain_state) {
    int rc = box_rows(b);
    if (rc) return rc;
    rc = pool_chain_init(ctx, dp, st);
    if (rc) return rc;
    b->chain_state = true;
    b->energy_ready = false;
  }
  if (!b->energy_ready) {
    int rc = box_rows(b);
    if (rc) return rc;
    rc = pool_system_energy(ctx, dp, true, st);
    if (rc) return rc;
    k_set_energy<<<1, 32, 0, st>>>(dp.P, dp.esum);
    CK(ctx, cudaGetLastError());
    b->energy_ready = true;
  }
  if (trace && n_steps > b->trace_cap) {
    if (b->dtrace) cudaFree(b->dtrace);
    b->dtrace = nullptr;
    CK(ctx, cudaMalloc((void**)&b->dtrace, sizeof(mcgpu_trace) * (size_t)n_steps));
    b->trace_cap = n_steps;
  }
  // one group for the chain: up to 16 warps (the wide kernel above 8); a
  // window of K steps: one such group per CTA of a K-CTA cluster, at least
  // K warps (one stages each step of the window)
  const int K = b->window;
  const int nw = std::max(K > 1 ? K : 1, std::min(16, dp.n_mol / 256));
  SmemShape sh = shape_for(dp.max_len, nw, pool_cache_n(dp));
  const int wsmem = K > 1 ? window_smem_bytes(sh, K) : 0;
  if (K > 1 && wsmem > kWindowSmemMax)
    return set_err(ctx, MCGPU_ERR_UNSUPPORTED, "a %d-step window needs %d B shared memory", K, wsmem);
  // with a Verlet list, short launches let stale lists be rebuilt promptly
  const int seg = dp.nl_on ? 64 : 1024;
  for (int done = 0; done < n_steps; done += seg) {
    const int k = std::min(seg, n_steps - done);
    int rc = pool_nl_rebuild(ctx, dp, st);
    if (rc) return rc;
    CK(ctx, cudaMemsetAsync(b->queue, 0, sizeof(unsigned), st));
    Pool P = dp.P;
    P.trace = nullptr;
    if (K > 1)
      CK(ctx, launch_chain_window(K, 1, nw * 32, wsmem, st, P, k, b->order, 1, sh,
                                  trace ? b->dtrace : nullptr, done, 0, 0));
    else if (nw > 8)
      k_chain_steps_wide<<<1, nw * 32, sh.bytes(), st>>>(P, k, b->queue, b->order, 1, nw, sh,
                                                         trace ? b->dtrace : nullptr, done, 0, 0);
    else
      k_chain_steps<<<1, nw * 32, sh.bytes(), st>>>(P, k, b->queue, b->order, 1, nw, sh,
                                                    trace ? b->dtrace : nullptr, done, 0, 0);
    CK(ctx, cudaGetLastError());
    b->rows_stale = true;
  }
  if (trace && n_steps > 0)
    CK(ctx, cudaMemcpyAsync(trace, b->dtrace, sizeof(mcgpu_trace) * (size_t)n_steps,
                            cudaMemcpyDeviceToHost, st));
  if (stats) {
    ChainHdr h;
    CK(ctx, cudaMemcpyAsync(&h, dh, sizeof(h), cudaMemcpyDeviceToHost, st));
    CK(ctx, cudaStreamSynchronize(st));
    stats->energy = h.energy;
    stats->steps = (int64_t)h.step;
    stats->accepted = h.accepted;
    stats->pairs = h.pairs;
    stats->error = h.error;
    stats->ties = h.ties;
    for (int k = 0; k < 3; k++) stats->box[k] = h.L[k];
    stats->vol_tried = h.vol_tried;
    stats->vol_accepted = h.vol_accepted;
    stats->nl_builds = h.nl_builds;
    stats->nl_full_scans = h.nl_full;
    stats->window_redo = h.win_redo;
  }
  CK(ctx, cudaStreamSynchronize(st));
  return MCGPU_OK;
}

// ---- batch ---------------------------------------------------------------------------

struct mcgpu_batch {
  mcgpu_ctx* ctx = nullptr;
  DevPool pool;
  unsigned* queue = nullptr;   // one counter per launch slot of a graph
  int* order = nullptr;
  int threads = 128, cpc = 1, spl = 16;  // CTA threads, chains per CTA, steps per launch
  int lanes = 0;                          // lanes per neighbour molecule cap (0 = per chain)
  int cache_n = 0;                        // shared-memory screen cache per group
  bool rows_stale = false;                // FP64 rows lag the chain state
  int max_slots = 0;
  cudaGraphExec_t graph = nullptr;
  int graph_launches = 0, graph_spl = 0, graph_threads = 0, graph_cpc = 0, graph_lanes = 0;
  int graph_interval = 0;                 // NPT interval the graph covers (0 = NVT graph)
  int window = 1;                         // steps per window (clusters of `window` CTAs)
  int graph_window = 0;
  // NPT: steps every chain has taken (all chains advance together), the
  // volume interval, and the volume phase's device buffers
  long long steps_done = 0;
  int vol_interval = 0;
  VolMove* vm = nullptr;
  double2* emol2 = nullptr;
  double2* eabs2 = nullptr;
  double2* vsum = nullptr;
  double2* vsum_abs = nullptr;
  int* vlist = nullptr;                   // chains of a re-take (3 * n_chains + 3)
  bool vol_has64 = false, vol_has32 = false;  // precisions of the NPT chains
  // snapshot for the autotuner
  std::vector<void*> snap;
};

static int batch_gwarps(const mcgpu_batch* bt) { return (bt->threads / 32) / bt->cpc; }

static int batch_grid(mcgpu_batch* bt, int* smem_out) {
  const int gw = batch_gwarps(bt);
  SmemShape sh = shape_for(bt->pool.max_len, gw, bt->cache_n);
  const int smem = sh.bytes() * bt->cpc;
  *smem_out = smem;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, bt->threads > 256 ? k_chain_steps_wide : k_chain_steps, bt->threads, smem);
  per_sm = std::max(per_sm, 1);
  const int need = (bt->pool.n_chains + bt->cpc - 1) / bt->cpc;
  return std::max(1, std::min(need, per_sm * bt->ctx->sm_count));
}

static int batch_launch(mcgpu_batch* bt, int steps, unsigned* q, cudaStream_t st,
                        mcgpu_trace* trace = nullptr, int trace_off = 0, int trace_stride = 0) {
  mcgpu_ctx* ctx = bt->ctx;
  int smem = 0;
  const int grid = batch_grid(bt, &smem);
  const int gw = batch_gwarps(bt);
  SmemShape sh = shape_for(bt->pool.max_len, gw, bt->cache_n);
  bt->rows_stale = true;
  int rc = pool_nl_rebuild(ctx, bt->pool, st);
  if (rc) return rc;
  CK(ctx, cudaMemsetAsync(q, 0, sizeof(unsigned), st));
  if (bt->window > 1) {
    const int K = bt->window, wsmem = window_smem_bytes(sh, K);
    const int n_cl = std::max(1, std::min(bt->pool.n_chains,
                                          window_max_clusters(K, bt->threads, wsmem)));
    CK(ctx, launch_chain_window(K, n_cl, bt->threads, wsmem, st, bt->pool.P, steps, bt->order,
                                bt->pool.n_chains, sh, trace, trace_off, trace_stride, bt->lanes));
    return MCGPU_OK;
  }
  if (bt->threads > 256)
    k_chain_steps_wide<<<grid, bt->threads, smem, st>>>(bt->pool.P, steps, q, bt->order,
                                                        bt->pool.n_chains, gw, sh, trace,
                                                        trace_off, trace_stride, bt->lanes);
  else
    k_chain_steps<<<grid, bt->threads, smem, st>>>(bt->pool.P, steps, q, bt->order,
                                                   bt->pool.n_chains, gw, sh, trace, trace_off,
                                                   trace_stride, bt->lanes);
  CK(ctx, cudaGetLastError());
  return MCGPU_OK;
}

extern "C" int mcgpu_batch_create(mcgpu_ctx* ctx, int n_chains, const mcgpu_box_desc* descs,
                                  const uint64_t* seeds, int rotation, mcgpu_batch** out) {
  if (!ctx || !descs || !seeds || !out) return set_err(ctx, MCGPU_ERR_INVALID, "null argument");
  *out = nullptr;
  if (n_chains <= 0) return set_err(ctx, MCGPU_ERR_INVALID, "n_chains %d must be > 0", n_chains);
  if (rotation != MCGPU_ROT_EULER && rotation != MCGPU_ROT_AXIS)
    return set_err(ctx, MCGPU_ERR_INVALID, "unknown rotation form %d", rotation);
  CK(ctx, cudaSetDevice(ctx->device));
  HostPool hp;
  if (int rc = build_pool(ctx, hp, descs, n_chains, seeds, rotation)) return rc;
  mcgpu_batch* bt = new mcgpu_batch();
  bt->ctx = ctx;
  int rc = upload_pool(ctx, hp, bt->pool);
  if (rc) {
    delete bt;
    return rc;
  }
  // Cost-descending task order (largest chains first): screen ~ n_mol,
  // pairs ~ max_len^2.
  std::vector<int> order(n_chains);
  for (int c = 0; c < n_chains; c++) order[c] = c;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b2) {
    const ChainHdr &ha = hp.hdr[a], &hb = hp.hdr[b2];
    return (double)ha.n_mol * (1 + ha.max_len) > (double)hb.n_mol * (1 + hb.max_len);
  });
  bt->max_slots = 64;
  cudaError_t e = cudaSuccess;
  bt->queue = dalloc<unsigned>(bt->max_slots, &e);
  bt->order = dalloc<int>(n_chains, &e);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(bt->order, order.data(), sizeof(int) * n_chains, cudaMemcpyHostToDevice,
                        ctx->stream);
  if (e != cudaSuccess) {
    mcgpu_batch_destroy(bt);
    return set_err(ctx, MCGPU_ERR_NOMEM, "batch allocation failed: %s", cudaGetErrorString(e));
  }
  bt->cache_n = pool_cache_n(bt->pool);
  // device-resident chain state (rows snapped to it), then the initial
  // running energies
  rc = pool_chain_init(ctx, bt->pool, ctx->stream);
  if (rc) {
    mcgpu_batch_destroy(bt);
    return rc;
  }
  // initial running energies: FP32-pair system energies (double-float
  // sums) over per-chain cell grids, the volume-move machinery at the
  // chains' own boxes; each chain's run_err starts at their error bound.
  // The chains compute in FP32 pairs throughout; FP64 enters where a
  // decision is too close to call.
  {
    cudaError_t e2 = cudaSuccess;
    Pool& P = bt->pool.P;
    const size_t nm = (size_t)bt->pool.n_mol;
    bt->vm = dalloc<VolMove>(n_chains, &e2);
    bt->emol2 = dalloc<double2>(nm, &e2);
    bt->eabs2 = dalloc<double2>(nm, &e2);
    bt->vsum = dalloc<double2>(n_chains, &e2);
    bt->vsum_abs = dalloc<double2>(n_chains, &e2);
    P.vc_cnt = dalloc<int>(nm, &e2);
    P.vc_start = dalloc<int>(nm, &e2);
    P.vc_mol = dalloc<int>(nm, &e2);
    P.vc_of = dalloc<int>(nm, &e2);
    if (e2 == cudaSuccess)
      e2 = launch_chain_energy(P, bt->pool.mol_chain, bt->pool.n_mol, bt->vm, bt->emol2, bt->eabs2,
                               bt->vsum, bt->vsum_abs, ctx->stream, MolRanges(), false);
    if (e2 == cudaSuccess) e2 = cudaStreamSynchronize(ctx->stream);
    if (e2 != cudaSuccess) {
      mcgpu_batch_destroy(bt);
      return set_err(ctx, MCGPU_ERR_CUDA, "initial energies: %s", cudaGetErrorString(e2));
    }
  }
  *out = bt;
  return MCGPU_OK;
}

static void batch_drop_graph(mcgpu_batch* bt) {
  if (bt->graph) cudaGraphExecDestroy(bt->graph);
  bt->graph = nullptr;
}

extern "C" int mcgpu_batch_destroy(mcgpu_batch* bt) {
  if (!bt) return MCGPU_OK;
  cudaSetDevice(bt->ctx->device);
  cudaStreamSynchronize(bt->ctx->stream);
  batch_drop_graph(bt);
  bt->pool.release();
  if (bt->queue) cudaFree(bt->queue);
  if (bt->order) cudaFree(bt->order);
  if (bt->vm) cudaFree(bt->vm);
  if (bt->emol2) cudaFree(bt->emol2);
  if (bt->eabs2) cudaFree(bt->eabs2);
  if (bt->vsum) cudaFree(bt->vsum);
  if (bt->vsum_abs) cudaFree(bt->vsum_abs);
  if (bt->vlist) cudaFree(bt->vlist);
  for (void* p : bt->snap)
    if (p) cudaFree(p);
  delete bt;
  return MCGPU_OK;
}

extern "C" int mcgpu_batch_set_tile(mcgpu_batch* bt, int threads, int cpc, int spl, int lanes) {
  if (!bt) return set_err(nullptr, MCGPU_ERR_INVALID, "null batch");
  mcgpu_ctx* ctx = bt->ctx;
  if (threads < 32 || threads > 512 || threads % 32)
    return set_err(ctx, MCGPU_ERR_INVALID, "threads %d must be a multiple of 32 in [32,512]", threads);
  if (cpc < 1 || (threads / 32) % cpc || (threads / 32) / cpc < 1)
    return set_err(ctx, MCGPU_ERR_INVALID, "chains per CTA %d must divide the CTA's %d warps", cpc,
                   threads / 32);
  if ((threads / 32) / cpc > 1 && cpc > 15)
    return set_err(ctx, MCGPU_ERR_INVALID, "at most 15 multi-warp groups per CTA");
  if (spl < 1) return set_err(ctx, MCGPU_ERR_INVALID, "steps per launch %d must be >= 1", spl);
  if (lanes != 0 && lanes != 1 && lanes != 2 && lanes != 4 && lanes != 8 && lanes != 16 && lanes != 32)
    return set_err(ctx, MCGPU_ERR_INVALID, "lanes per molecule %d must be 0 or a power of two <= 32",
                   lanes);
  int smem = shape_for(bt->pool.max_len, (threads / 32) / cpc, bt->cache_n).bytes() * cpc;
  if (smem > 200 * 1024) return set_err(ctx, MCGPU_ERR_UNSUPPORTED, "tile needs %d B shared memory", smem);
  if (bt->window > 1 && (cpc != 1 || threads / 32 < bt->window))
    return set_err(ctx, MCGPU_ERR_INVALID,
                   "the batch runs %d-step windows (one chain per CTA, at least %d warps): set the "
                   "window to 1 first", bt->window, bt->window);
  if (bt->window > 1 &&
      window_smem_bytes(shape_for(bt->pool.max_len, threads / 32, bt->cache_n), bt->window) >
          kWindowSmemMax)
    return set_err(ctx, MCGPU_ERR_UNSUPPORTED, "tile too large for a %d-step window", bt->window);
  bt->threads = threads;
  bt->cpc = cpc;
  bt->spl = spl;
  bt->lanes = lanes;
  batch_drop_graph(bt);
  return MCGPU_OK;
}

// Window sizes the windowed chain kernel takes (they divide the 32 moves
// drawn at a time; 16 is a non-portable cluster size).
static bool window_size_ok(int k) { return k == 1 || k == 2 || k == 4 || k == 8 || k == 16; }

extern "C" int mcgpu_batch_set_window(mcgpu_batch* bt, int k) {
  if (!bt) return set_err(nullptr, MCGPU_ERR_INVALID, "null batch");
  mcgpu_ctx* ctx = bt->ctx;
  if (!window_size_ok(k)) return set_err(ctx, MCGPU_ERR_INVALID, "window %d must be 1, 2, 4, 8 or 16", k);
  if (k > 1) {
    if (bt->cpc != 1)
      return set_err(ctx, MCGPU_ERR_INVALID, "a window needs one chain per CTA (tile has %d)", bt->cpc);
    if (bt->threads / 32 < k)
      return set_err(ctx, MCGPU_ERR_INVALID, "a %d-step window needs at least %d warps per CTA", k, k);
    const SmemShape sh = shape_for(bt->pool.max_len, bt->threads / 32, bt->cache_n);
    const int wsmem = window_smem_bytes(sh, k);
    if (wsmem > kWindowSmemMax)
      return set_err(ctx, MCGPU_ERR_UNSUPPORTED, "a %d-step window needs %d B shared memory", k, wsmem);
    if (window_max_clusters(k, bt->threads, wsmem) < 1)
      return set_err(ctx, MCGPU_ERR_UNSUPPORTED, "no cluster of %d CTAs of %d threads fits the device",
                     k, bt->threads);
  }
  bt->window = k;
  batch_drop_graph(bt);
  return MCGPU_OK;
}

extern "C" int mcgpu_chain_set_window(mcgpu_box* b, int k) {
  if (!b) return set_err(nullptr, MCGPU_ERR_INVALID, "null box");
  if (!window_size_ok(k)) return set_err(b->ctx, MCGPU_ERR_INVALID, "window %d must be 1, 2, 4, 8 or 16", k);
  if (k > 1) {
    const int nw = std::max(k, std::min(16, b->pool.n_mol / 256));
    const SmemShape sh = shape_for(b->pool.max_len, nw, pool_cache_n(b->pool));
    const int wsmem = window_smem_bytes(sh, k);
    if (wsmem > kWindowSmemMax)
      return set_err(b->ctx, MCGPU_ERR_UNSUPPORTED, "a %d-step window needs %d B shared memory", k,
                     wsmem);
    if (window_max_clusters(k, nw * 32, wsmem) < 1)
      return set_err(b->ctx, MCGPU_ERR_UNSUPPORTED, "no cluster of %d CTAs of %d threads fits the device",
                     k, nw * 32);
  }
  b->window = k;
  return MCGPU_OK;
}

extern "C" int mcgpu_batch_get_tile(mcgpu_batch* bt, int* threads, int* cpc, int* spl, int* lanes) {
  if (!bt) return set_err(nullptr, MCGPU_ERR_INVALID, "null batch");
  if (threads) *threads = bt->threads;
  if (cpc) *cpc = bt->cpc;
  if (spl) *spl = bt->spl;
  if (lanes) *lanes = bt->lanes;
  return MCGPU_OK;
}

// Captures `launches` launches of spl steps each into a graph (one queue
// counter per launch, reset by a memset node).  With interval > 0 the graph
// is one NPT interval instead: launches covering `interval` steps, then the
// volume phase.
static int batch_build_graph(mcgpu_batch* bt, int launches, int interval) {
  mcgpu_ctx* ctx = bt->ctx;
  batch_drop_graph(bt);
  cudaStream_t st = ctx->stream;
  cudaGraph_t g = nullptr;
  CK(ctx, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  int rc = MCGPU_OK;
  if (interval > 0) {
    int done = 0;
    for (int l = 0; done < interval && rc == MCGPU_OK; l++) {
      const int k = std::min(bt->spl, interval - done);
      rc = batch_launch(bt, k, bt->queue + l, st);
      done += k;
    }
    if (rc == MCGPU_OK) {
      cudaError_t e = launch_volume_phase(bt->pool.P, bt->pool.mol_chain, bt->pool.n_mol, bt->vm,
                                          bt->emol2, bt->eabs2, bt->vsum, bt->vsum_abs, bt->vlist,
                                          nullptr, 0,
                                          0, st, MolRanges(), bt->vol_has64, bt->vol_has32);
      if (e != cudaSuccess) rc = set_err(ctx, MCGPU_ERR_CUDA, "volume phase launch: %s", cudaGetErrorString(e));
    }
  } else {
    for (int l = 0; l < launches && rc == MCGPU_OK; l++) rc = batch_launch(bt, bt->spl, bt->queue + l, st);
  }
  cudaError_t e = cudaStreamEndCapture(st, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return set_err(ctx, MCGPU_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
  e = cudaGraphInstantiate(&bt->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return set_err(ctx, MCGPU_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
  bt->graph_launches = launches;
  bt->graph_spl = bt->spl;
  bt->graph_threads = bt->threads;
  bt->graph_cpc = bt->cpc;
  bt->graph_lanes = bt->lanes;
  bt->graph_interval = interval;
  bt->graph_window = bt->window;
  return MCGPU_OK;
}

static bool batch_graph_matches(const mcgpu_batch* bt, int launches, int interval) {
  return bt->graph && bt->graph_spl == bt->spl && bt->graph_launches == launches &&
         bt->graph_threads == bt->threads && bt->graph_cpc == bt->cpc &&
         bt->graph_lanes == bt->lanes && bt->graph_interval == interval &&
         bt->graph_window == bt->window;
}

// Steps n_steps with direct launches of at most spl steps (recording steps
// at trace[c * trace_stride + trace_off + s] when trace is non-null).
static int batch_steps_direct(mcgpu_batch* bt, int n_steps, mcgpu_trace* trace, int trace_off,
                              int trace_stride) {
  for (int done = 0; done < n_steps;) {
    const int k = std::min(bt->spl, n_steps - done);
    int rc = batch_launch(bt, k, bt->queue + ((done / bt->spl) % bt->max_slots), bt->ctx->stream,
                          trace, trace_off + done, trace_stride);
    if (rc) return rc;
    done += k;
  }
  return MCGPU_OK;
}

// Advances every chain by n_steps: NVT in graph replays of 32 launches
// where possible; NPT interval by interval, each followed by the volume
// phase (one graph per interval when no trace is recorded).
static int batch_advance(mcgpu_batch* bt, int n_steps, mcgpu_trace* trace, int trace_stride,
                         mcgpu_vol_trace* vtrace, int vstride) {
  mcgpu_ctx* ctx = bt->ctx;
  const int spl = bt->spl;
  const int iv = bt->vol_interval;
  // graph replays do not pass through batch_launch: mark the FP64 rows
  // stale here for every path
  if (n_steps > 0) bt->rows_stale = true;
  if (iv <= 0) {
    const int full = n_steps / spl;
    const int per_graph = std::min(bt->max_slots, 32);
    int done = 0;
    if (!trace && full >= per_graph) {
      if (!batch_graph_matches(bt, per_graph, 0)) {
        int rc = batch_build_graph(bt, per_graph, 0);
        if (rc) return rc;
      }
      while (full - done >= per_graph) {
        CK(ctx, cudaGraphLaunch(bt->graph, ctx->stream));
        done += per_graph;
      }
    }
    int rc = batch_steps_direct(bt, n_steps - done * spl, trace, done * spl, trace_stride);
    if (rc) return rc;
    bt->steps_done += n_steps;
    return MCGPU_OK;
  }
  const int launches_per_interval = (iv + spl - 1) / spl;
  const bool graphable = !trace && !vtrace && launches_per_interval <= bt->max_slots;
  int done = 0, vk = 0;
  while (done < n_steps) {
    const int phase = (int)(bt->steps_done % iv);
    if (phase == 0 && n_steps - done >= iv && graphable) {
      if (!batch_graph_matches(bt, launches_per_interval, iv)) {
        int rc = batch_build_graph(bt, launches_per_interval, iv);
        if (rc) return rc;
      }
      CK(ctx, cudaGraphLaunch(bt->graph, ctx->stream));
      done += iv;
      bt->steps_done += iv;
      continue;
    }
    const int seg = std::min(n_steps - done, iv - phase);
    int rc = batch_steps_direct(bt, seg, trace, done, trace_stride);
    if (rc) return rc;
    done += seg;
    bt->steps_done += seg;
    if (bt->steps_done % iv == 0) {
      CK(ctx, launch_volume_phase(bt->pool.P, bt->pool.mol_chain, bt->pool.n_mol, bt->vm, bt->emol2,
                                  bt->eabs2, bt->vsum, bt->vsum_abs, bt->vlist, vtrace, vk, vstride,
                                  ctx->stream, MolRanges(), bt->vol_has64, bt->vol_has32));
      vk++;
    }
  }
  return MCGPU_OK;
}

extern "C" int mcgpu_batch_run(mcgpu_batch* bt, int n_steps, int sync) {
  if (!bt) return set_err(nullptr, MCGPU_ERR_INVALID, "null batch");
  mcgpu_ctx* ctx = bt->ctx;
  if (n_steps < 0) return set_err(ctx, MCGPU_ERR_INVALID, "negative step count");
  int rc = batch_advance(bt, n_steps, nullptr, 0, nullptr, 0);
  if (rc) return rc;
  if (sync) CK(ctx, cudaStreamSynchronize(ctx->stream));
  return MCGPU_OK;
}

extern "C" int mcgpu_batch_run_traced(mcgpu_batch* bt, int n_steps, mcgpu_trace* out,
                                      mcgpu_vol_trace* vol_out) {
  if (!bt || !out) return set_err(bt ? bt->ctx : nullptr, MCGPU_ERR_INVALID, "null argument");
  mcgpu_ctx* ctx = bt->ctx;
  if (n_steps <= 0) return set_err(ctx, MCGPU_ERR_INVALID, "step count %d must be > 0", n_steps);
  const size_t n = (size_t)n_steps * bt->pool.n_chains;
  const int vstride = bt->vol_interval > 0 ? n_steps / bt->vol_interval + 1 : 0;
  const size_t nv = (size_t)vstride * bt->pool.n_chains;
  mcgpu_trace* d = nullptr;
  mcgpu_vol_trace* dv = nullptr;
  CK(ctx, cudaMalloc((void**)&d, sizeof(mcgpu_trace) * n));
  cudaError_t e = cudaSuccess;
  if (vol_out && nv > 0) {
    e = cudaMalloc((void**)&dv, sizeof(mcgpu_vol_trace) * nv);
    if (e == cudaSuccess) e = cudaMemsetAsync(dv, 0, sizeof(mcgpu_vol_trace) * nv, ctx->stream);
  }
  int rc = MCGPU_OK;
  if (e == cudaSuccess) rc = batch_advance(bt, n_steps, d, n_steps, dv, vstride);
  if (rc == MCGPU_OK && e == cudaSuccess)
    e = cudaMemcpyAsync(out, d, sizeof(mcgpu_trace) * n, cudaMemcpyDeviceToHost, ctx->stream);
  if (rc == MCGPU_OK && e == cudaSuccess && dv)
    e = cudaMemcpyAsync(vol_out, dv, sizeof(mcgpu_vol_trace) * nv, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(d);
  if (dv) cudaFree(dv);
  if (rc) return rc;
  if (e != cudaSuccess) return set_err(ctx, MCGPU_ERR_CUDA, "traced run failed: %s", cudaGetErrorString(e));
  return MCGPU_OK;
}

extern "C" int mcgpu_batch_set_verlet(mcgpu_batch* bt, double skin) {
  if (!bt) return set_err(nullptr, MCGPU_ERR_INVALID, "null batch");
  if (!std::isfinite(skin)) return set_err(bt->ctx, MCGPU_ERR_INVALID, "skin %g", skin);
  batch_drop_graph(bt);
  return pool_set_verlet(bt->ctx, bt->pool, skin, bt->ctx->stream);
}

extern "C" int mcgpu_batch_set_lrc(mcgpu_batch* bt, const double* lrc_v) {
  if (!bt || !lrc_v) return set_err(bt ? bt->ctx : nullptr, MCGPU_ERR_INVALID, "null argument");
  mcgpu_ctx* ctx = bt->ctx;
  const int n = bt->pool.n_chains;
  for (int c = 0; c < n; c++)
    if (!std::isfinite(lrc_v[c]))
      return set_err(ctx, MCGPU_ERR_INVALID, "lrc_v[%d] is not finite", c);
  // one strided copy into the lrc_v field of every device header
  CK(ctx, cudaMemcpy2DAsync((char*)bt->pool.P.hdr + offsetof(ChainHdr, lrc_v), sizeof(ChainHdr),
                            lrc_v, sizeof(double), sizeof(double), (size_t)n,
                            cudaMemcpyHostToDevice, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  for (int c = 0; c < n; c++) bt->pool.hdr[c].lrc_v = lrc_v[c];
  return MCGPU_OK;
}

extern "C" int mcgpu_box_set_verlet(mcgpu_box* b, double skin) {
  if (!b) return set_err(nullptr, MCGPU_ERR_INVALID, "null box");
  if (!std::isfinite(skin)) return set_err(b->ctx, MCGPU_ERR_INVALID, "skin %g", skin);
  return pool_set_verlet(b->ctx, b->pool, skin, b->ctx->stream);
}

extern "C" int mcgpu_batch_set_npt(mcgpu_batch* bt, int interval, const double* pressure_atm,
                                   const double* max_dlnv, int precision) {
  if (!bt) return set_err(nullptr, MCGPU_ERR_INVALID, "null batch");
  mcgpu_ctx* ctx = bt->ctx;
  const int nc = bt->pool.n_chains;
  if (interval < 0) return set_err(ctx, MCGPU_ERR_INVALID, "volume interval %d must be >= 0", interval);
  if (precision != MCGPU_PREC_FP64 && precision != MCGPU_PREC_MIXED)
    return set_err(ctx, MCGPU_ERR_INVALID, "unknown volume-move precision %d", precision);
  const int mixed = interval > 0 && precision == MCGPU_PREC_MIXED;
  std::vector<double> p(nc, 0.0), dl(nc, 0.0);
  std::vector<int> iv(nc, interval), vmx(nc, mixed);
  if (interval > 0) {
    if (!pressure_atm || !max_dlnv) return set_err(ctx, MCGPU_ERR_INVALID, "null NPT parameters");
    for (int c = 0; c < nc; c++) {
      if (!std::isfinite(pressure_atm[c]) || pressure_atm[c] < 0)
        return set_err(ctx, MCGPU_ERR_INVALID, "chain %d: pressure %g atm", c, pressure_atm[c]);
      if (!(max_dlnv[c] > 0 && max_dlnv[c] <= 0.1))
        return set_err(ctx, MCGPU_ERR_INVALID, "chain %d: max ln V step %g outside (0, 0.1]", c,
                       max_dlnv[c]);
      p[c] = pressure_atm[c] * kAtmKcal;
      dl[c] = max_dlnv[c];
    }
    cudaError_t e = cudaSuccess;
    if (!bt->vm) bt->vm = dalloc<VolMove>(nc, &e);
    if (!bt->emol2) bt->emol2 = dalloc<double2>(bt->pool.n_mol, &e);
    if (!bt->eabs2) bt->eabs2 = dalloc<double2>(bt->pool.n_mol, &e);
    if (!bt->vsum) bt->vsum = dalloc<double2>(nc, &e);
    if (!bt->vsum_abs) bt->vsum_abs = dalloc<double2>(nc, &e);
    if (!bt->vlist) bt->vlist = dalloc<int>(3 * (size_t)nc + 3, &e);
    Pool& P = bt->pool.P;
    if (!P.vc_cnt) {
      const size_t nm = (size_t)bt->pool.n_mol;
      P.vc_cnt = dalloc<int>(nm, &e);
      P.vc_start = dalloc<int>(nm, &e);
      P.vc_mol = dalloc<int>(nm, &e);
      P.vc_of = dalloc<int>(nm, &e);
    }
    if (e != cudaSuccess) return set_err(ctx, MCGPU_ERR_NOMEM, "NPT buffers: %s", cudaGetErrorString(e));
  }
  cudaStream_t st = ctx->stream;
  ChainHdr* h = bt->pool.P.hdr;
  CK(ctx, cudaMemcpy2DAsync(&h->pressure, sizeof(ChainHdr), p.data(), sizeof(double), sizeof(double),
                            nc, cudaMemcpyHostToDevice, st));
  CK(ctx, cudaMemcpy2DAsync(&h->max_dlnv, sizeof(ChainHdr), dl.data(), sizeof(double), sizeof(double),
                            nc, cudaMemcpyHostToDevice, st));
  CK(ctx, cudaMemcpy2DAsync(&h->vol_interval, sizeof(ChainHdr), iv.data(), sizeof(int), sizeof(int),
                            nc, cudaMemcpyHostToDevice, st));
  CK(ctx, cudaMemcpy2DAsync(&h->vol_mixed, sizeof(ChainHdr), vmx.data(), sizeof(int), sizeof(int),
                            nc, cudaMemcpyHostToDevice, st));
  CK(ctx, cudaStreamSynchronize(st));
  bt->vol_interval = interval;
  bt->vol_has64 = interval > 0 && !mixed;
  bt->vol_has32 = mixed;
  batch_drop_graph(bt);
  return MCGPU_OK;
}

extern "C" int mcgpu_batch_set_precision(mcgpu_batch* bt, int precision) {
  if (!bt) return set_err(nullptr, MCGPU_ERR_INVALID, "null batch");
  mcgpu_ctx* ctx = bt->ctx;
  if (precision != MCGPU_PREC_FP64 && precision != MCGPU_PREC_MIXED)
    return set_err(ctx, MCGPU_ERR_INVALID, "unknown pair precision %d", precision);
  const int nc = bt->pool.n_chains;
  std::vector<int> v(nc, precision == MCGPU_PREC_FP64 ? 1 : 0);
  CK(ctx, cudaMemcpy2DAsync(&bt->pool.P.hdr->fp64_pairs, sizeof(ChainHdr), v.data(), sizeof(int),
                            sizeof(int), nc, cudaMemcpyHostToDevice, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return MCGPU_OK;
}

extern "C" int mcgpu_batch_sync(mcgpu_batch* bt) {
  if (!bt) return set_err(nullptr, MCGPU_ERR_INVALID, "null batch");
  CK(bt->ctx, cudaStreamSynchronize(bt->ctx->stream));
  return MCGPU_OK;
}

extern "C" int mcgpu_batch_stats(mcgpu_batch* bt, mcgpu_chain_stats* stats) {
  if (!bt || !stats) return set_err(bt ? bt->ctx : nullptr, MCGPU_ERR_INVALID, "null argument");
  mcgpu_ctx* ctx = bt->ctx;
  std::vector<ChainHdr> h(bt->pool.n_chains);
  CK(ctx, cudaMemcpyAsync(h.data(), bt->pool.P.hdr, sizeof(ChainHdr) * h.size(),
                          cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  int err = 0;
  for (size_t c = 0; c < h.size(); c++) {
    stats[c].energy = h[c].energy;
    stats[c].steps = (int64_t)h[c].step;
    stats[c].accepted = h[c].accepted;
    stats[c].pairs = h[c].pairs;
    stats[c].error = h[c].error;
    stats[c].ties = h[c].ties;
    for (int k = 0; k < 3; k++) stats[c].box[k] = h[c].L[k];
    stats[c].vol_tried = h[c].vol_tried;
    stats[c].vol_accepted = h[c].vol_accepted;
    stats[c].nl_builds = h[c].nl_builds;
    stats[c].nl_full_scans = h[c].nl_full;
    stats[c].window_redo = h[c].win_redo;
    err |= h[c].error;
  }
  if (err) return set_err(ctx, MCGPU_ERR_DEVICE, "a chain reported device error status %d", err);
  return MCGPU_OK;
}

extern "C" int mcgpu_batch_download(mcgpu_batch* bt, int chain, double* x, double* y, double* z) {
  if (!bt || !x || !y || !z) return set_err(bt ? bt->ctx : nullptr, MCGPU_ERR_INVALID, "null argument");
  mcgpu_ctx* ctx = bt->ctx;
  if (chain < 0 || chain >= bt->pool.n_chains)
    return set_err(ctx, MCGPU_ERR_INVALID, "chain %d out of [0,%d)", chain, bt->pool.n_chains);
  if (bt->rows_stale) {
    int rc = pool_chain_export(ctx, bt->pool, ctx->stream);
    if (rc) return rc;
    bt->rows_stale = false;
  }
  const ChainHdr& h = bt->pool.hdr[chain];
  const size_t n = (size_t)h.n_atom;
  CK(ctx, cudaMemcpyAsync(x, bt->pool.P.x + h.atom0, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaMemcpyAsync(y, bt->pool.P.y + h.atom0, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaMemcpyAsync(z, bt->pool.P.z + h.atom0, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return MCGPU_OK;
}

extern "C" int mcgpu_batch_download_all(mcgpu_batch* bt, double* x, double* y, double* z) {
  if (!bt || !x || !y || !z) return set_err(bt ? bt->ctx : nullptr, MCGPU_ERR_INVALID, "null argument");
  mcgpu_ctx* ctx = bt->ctx;
  if (bt->rows_stale) {
    int rc = pool_chain_export(ctx, bt->pool, ctx->stream);
    if (rc) return rc;
    bt->rows_stale = false;
  }
  const size_t n = (size_t)bt->pool.n_atom;
  CK(ctx, cudaMemcpyAsync(x, bt->pool.P.x, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaMemcpyAsync(y, bt->pool.P.y, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaMemcpyAsync(z, bt->pool.P.z, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return MCGPU_OK;
}

extern "C" int mcgpu_batch_system_energy(mcgpu_batch* bt, double* out) {
  if (!bt || !out) return set_err(bt ? bt->ctx : nullptr, MCGPU_ERR_INVALID, "null argument");
  mcgpu_ctx* ctx = bt->ctx;
  if (bt->rows_stale) {
    int rc = pool_chain_export(ctx, bt->pool, ctx->stream);
    if (rc) return rc;
    bt->rows_stale = false;
  }
  int rc = pool_system_energy(ctx, bt->pool, true, ctx->stream);
  if (rc) return rc;
  CK(ctx, cudaMemcpyAsync(out, bt->pool.esum, sizeof(double) * bt->pool.n_chains,
                          cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return MCGPU_OK;
}

// ---- checkpoint / restore -----------------------------------------------------------

namespace {

struct CkptHead {
  char magic[8];
  uint32_t version, n_chains, n_mol, n_atom, n_pidx, nl_stride, nl_on, vol_interval;
  int64_t steps_done;
  uint64_t layout, payload, checksum, hdr_bytes;
};
constexpr char kCkptMagic[8] = {'M', 'C', 'G', 'P', 'U', 'C', 'K', '1'};

uint64_t fnv1a(uint64_t h, const void* p, size_t n) {
  const unsigned char* b = (const unsigned char*)p;
  for (size_t i = 0; i < n; i++) h = (h ^ b[i]) * 1099511628211ull;
  return h;
}

// Pool layout a checkpoint belongs to: molecule ranges and chain offsets.
uint64_t pool_layout(const DevPool& dp) {
  uint64_t h = 1469598103934665603ull;
  h = fnv1a(h, dp.mstart.data(), dp.mstart.size() * sizeof(int));
  h = fnv1a(h, dp.mlen.data(), dp.mlen.size() * sizeof(int));
  for (const ChainHdr& c : dp.hdr) {
    const int v[] = {c.atom0, c.mol0, c.pidx0, c.n_mol, c.n_atom, c.n_pidx, c.max_len};
    h = fnv1a(h, v, sizeof(v));
  }
  return h;
}

struct CkptRow {
  void* p;
  size_t bytes;
};

// Device rows a run changes, in blob order.
std::vector<CkptRow> ckpt_rows(const DevPool& dp) {
  std::vector<CkptRow> r = {
      {dp.P.x, 8ull * dp.n_atom},     {dp.P.y, 8ull * dp.n_atom},
      {dp.P.z, 8ull * dp.n_atom},     {dp.P.aoff, 16ull * dp.n_atom},
      {dp.P.mfix, 16ull * dp.n_mol},  {dp.P.mq, 16ull * dp.n_mol},
      {dp.P.ppos, 16ull * dp.n_pidx}, {dp.P.hdr, sizeof(ChainHdr) * (size_t)dp.n_chains}};
  if (dp.nl_on) {
    r.push_back({dp.P.nl, 4ull * dp.n_mol * (size_t)dp.P.nl_stride});
    r.push_back({dp.P.nl_cnt, 4ull * dp.n_mol});
    r.push_back({dp.P.pbuild, 16ull * dp.n_pidx});
  }
  return r;
}

}  // namespace

extern "C" int mcgpu_batch_checkpoint(mcgpu_batch* bt, void* buf, size_t cap, size_t* used) {
  if (!bt || !used) return set_err(bt ? bt->ctx : nullptr, MCGPU_ERR_INVALID, "null argument");
  mcgpu_ctx* ctx = bt->ctx;
  DevPool& dp = bt->pool;
  const std::vector<CkptRow> rows = ckpt_rows(dp);
  size_t payload = 0;
  for (const CkptRow& r : rows) payload += r.bytes;
  *used = sizeof(CkptHead) + payload;
  if (!buf) return MCGPU_OK;
  if (cap < *used)
    return set_err(ctx, MCGPU_ERR_INVALID, "checkpoint needs %zu bytes, buffer has %zu", *used, cap);
  if (bt->rows_stale) {
    int rc = pool_chain_export(ctx, dp, ctx->stream);
    if (rc) return rc;
    bt->rows_stale = false;
  }
  char* out = (char*)buf + sizeof(CkptHead);
  for (const CkptRow& r : rows) {
    CK(ctx, cudaMemcpyAsync(out, r.p, r.bytes, cudaMemcpyDeviceToHost, ctx->stream));
    out += r.bytes;
  }
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  CkptHead h{};
  std::memcpy(h.magic, kCkptMagic, 8);
  h.version = 1;
  h.n_chains = (uint32_t)dp.n_chains;
  h.n_mol = (uint32_t)dp.n_mol;
  h.n_atom = (uint32_t)dp.n_atom;
  h.n_pidx = (uint32_t)dp.n_pidx;
  h.nl_stride = dp.nl_on ? (uint32_t)dp.P.nl_stride : 0u;
  h.nl_on = dp.nl_on ? 1u : 0u;
  h.vol_interval = (uint32_t)bt->vol_interval;
  h.steps_done = bt->steps_done;
  h.layout = pool_layout(dp);
  h.payload = payload;
  h.hdr_bytes = sizeof(ChainHdr);
  h.checksum = fnv1a(1469598103934665603ull, (const char*)buf + sizeof(CkptHead), payload);
  std::memcpy(buf, &h, sizeof(h));
  return MCGPU_OK;
}

extern "C" int mcgpu_batch_restore(mcgpu_batch* bt, const void* buf, size_t len) {
  if (!bt || !buf) return set_err(bt ? bt->ctx : nullptr, MCGPU_ERR_INVALID, "null argument");
  mcgpu_ctx* ctx = bt->ctx;
  DevPool& dp = bt->pool;
  CkptHead h;
  if (len < sizeof(h)) return set_err(ctx, MCGPU_ERR_INVALID, "checkpoint too short");
  std::memcpy(&h, buf, sizeof(h));
  if (std::memcmp(h.magic, kCkptMagic, 8) != 0 || h.version != 1)
    return set_err(ctx, MCGPU_ERR_INVALID, "not a checkpoint of this library");
  if (h.hdr_bytes != sizeof(ChainHdr) || h.n_chains != (uint32_t)dp.n_chains ||
      h.n_mol != (uint32_t)dp.n_mol || h.n_atom != (uint32_t)dp.n_atom ||
      h.n_pidx != (uint32_t)dp.n_pidx || h.layout != pool_layout(dp))
    return set_err(ctx, MCGPU_ERR_INVALID, "checkpoint of another batch layout");
  if (h.nl_on != (dp.nl_on ? 1u : 0u) || (dp.nl_on && h.nl_stride != (uint32_t)dp.P.nl_stride))
    return set_err(ctx, MCGPU_ERR_INVALID,
                   "checkpoint Verlet setting differs (set the same skin before restoring)");
  if (h.vol_interval != (uint32_t)bt->vol_interval)
    return set_err(ctx, MCGPU_ERR_INVALID,
                   "checkpoint NPT interval %u, batch %d (set_npt before restoring)",
                   h.vol_interval, bt->vol_interval);
  const std::vector<CkptRow> rows = ckpt_rows(dp);
  size_t payload = 0;
  for (const CkptRow& r : rows) payload += r.bytes;
  if (h.payload != payload || len < sizeof(h) + payload)
    return set_err(ctx, MCGPU_ERR_INVALID, "checkpoint payload size mismatch");
  const char* in = (const char*)buf + sizeof(h);
  if (fnv1a(1469598103934665603ull, in, payload) != h.checksum)
    return set_err(ctx, MCGPU_ERR_INVALID, "checkpoint checksum mismatch");
  for (const CkptRow& r : rows) {
    CK(ctx, cudaMemcpyAsync(r.p, in, r.bytes, cudaMemcpyHostToDevice, ctx->stream));
    in += r.bytes;
  }
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  bt->steps_done = h.steps_done;
  bt->rows_stale = false;
  return MCGPU_OK;
}

// ---- autotuner ---------------------------------------------------------------------

// Device-side copy of the rows a checkpoint holds (the Verlet lists
// included, so a restored batch never screens with lists of another state).
static int batch_snapshot(mcgpu_batch* bt, bool restore) {
  mcgpu_ctx* ctx = bt->ctx;
  const std::vector<CkptRow> rows = ckpt_rows(bt->pool);
  const int nr = (int)rows.size();
  if (!restore) {
    for (void* p : bt->snap)
      if (p) cudaFree(p);
    bt->snap.assign(nr, nullptr);
    for (int r = 0; r < nr; r++) CK(ctx, cudaMalloc(&bt->snap[r], rows[r].bytes));
  } else if ((int)bt->snap.size() != nr) {
    return set_err(ctx, MCGPU_ERR_INVALID, "snapshot taken with other Verlet settings");
  }
  for (int r = 0; r < nr; r++) {
    if (restore)
      CK(ctx, cudaMemcpyAsync(rows[r].p, bt->snap[r], rows[r].bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    else
      CK(ctx, cudaMemcpyAsync(bt->snap[r], rows[r].p, rows[r].bytes, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  return MCGPU_OK;
}

extern "C" int mcgpu_batch_autotune(mcgpu_batch* bt, int trial_steps) {
  if (!bt) return set_err(nullptr, MCGPU_ERR_INVALID, "null batch");
  mcgpu_ctx* ctx = bt->ctx;
  if (trial_steps < 1) trial_steps = 64;
  if (bt->window > 1)
    return set_err(ctx, MCGPU_ERR_INVALID, "the tile search times one-step kernels: set the window to 1 first");
  int rc = batch_snapshot(bt, false);
  if (rc) return rc;
  const long long steps0 = bt->steps_done;
  struct Tile { int threads, cpc, spl, lanes; };
  cudaEvent_t e0, e1;
  CK(ctx, cudaEventCreate(&e0));
  CK(ctx, cudaEventCreate(&e1));
  // Every timed launch starts with L2 cleared (a write of twice its size),
  // as it does for a state larger than L2 or a batch run between other
  // work; without the scratch buffer the launches run as they come.
  int l2 = 0;
  cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, ctx->device);
  void* flush = nullptr;
  const size_t flush_bytes = 2 * (size_t)std::max(l2, 0);
  if (flush_bytes && cudaMalloc(&flush, flush_bytes) != cudaSuccess) {
    flush = nullptr;
    cudaGetLastError();
  }
  // time of trial_steps steps with tile T from the saved state: the fastest
  // of three timed runs after a warm-up launch (per-step cost, so runs longer
  // than trial_steps are scaled)
  auto trial = [&](const Tile& T, float* out) -> int {
    *out = 1e30f;
    if (mcgpu_batch_set_tile(bt, T.threads, T.cpc, T.spl, T.lanes) != MCGPU_OK) return MCGPU_OK;
    int r = batch_snapshot(bt, true);
    if (r) return r;
    bt->steps_done = steps0;
    r = mcgpu_batch_run(bt, T.spl, 0);
    if (r) return r;
    const int n = std::max(trial_steps, 2 * T.spl);
    for (int rep = 0; rep < 3; rep++) {
      float total = 0;
      for (int done = 0; done < n; done += T.spl) {
        if (flush) CK(ctx, cudaMemsetAsync(flush, rep + 1, flush_bytes, ctx->stream));
        CK(ctx, cudaEventRecord(e0, ctx->stream));
        r = mcgpu_batch_run(bt, std::min(T.spl, n - done), 0);
        if (r) return r;
        CK(ctx, cudaEventRecord(e1, ctx->stream));
        CK(ctx, cudaEventSynchronize(e1));
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        total += ms;
      }
      *out = std::min(*out, total * (float)trial_steps / (float)n);
    }
    return MCGPU_OK;
  };
  float best = 1e30f, ms = 0;
  Tile bestT = {bt->threads, bt->cpc, bt->spl, bt->lanes};
  // CTA shape (threads, chains per CTA) and lanes per neighbour molecule
  // together (the best width depends on the lanes), at 64 steps a launch
  // (shorter launches weigh the launch tail, which the final steps-per-launch
  // search settles)
  std::vector<Tile> shapes;
  const int tw[] = {64, 128, 256, 512};
  for (int t : tw)
    for (int gw = 1; gw <= t / 32; gw *= 2) {
      const int cpc = (t / 32) / gw;
      if (gw > 1 && cpc > 15) continue;
      // 512 threads only as one 16-warp group (smaller groups repeat the
      // 256-thread shapes with fewer CTAs per SM)
      if (t == 512 && cpc != 1) continue;
      shapes.push_back({t, cpc, 64, 0});
    }
  // one group of 3, 5, 6 or 7 warps per CTA (at 128 registers a thread,
  // 5-warp CTAs fit three to an SM: three chains in flight instead of two)
  for (int t : {96, 160, 192, 224}) shapes.push_back({t, 1, 64, 0});
  int max_tpm = 1;
  for (const ChainHdr& h : bt->pool.hdr) max_tpm = std::max(max_tpm, h.tpm);
  for (const Tile& S : shapes)
    for (int lanes = 0; lanes < max_tpm && rc == MCGPU_OK; lanes = lanes ? lanes << 1 : 1) {
      const Tile T = {S.threads, S.cpc, S.spl, lanes};
      rc = trial(T, &ms);
      if (rc == MCGPU_OK && ms < best) {
        best = ms;
        bestT = T;
      }
    }
  // steps per launch for the best shape
  const int spls[] = {4, 16, 64};
  for (int spl : spls) {
    if (rc) break;
    const Tile T = {bestT.threads, bestT.cpc, spl, bestT.lanes};
    rc = trial(T, &ms);
    if (rc == MCGPU_OK && ms <= best) {
      best = ms;
      bestT = T;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (flush) cudaFree(flush);
  if (rc) return rc;
  rc = mcgpu_batch_set_tile(bt, bestT.threads, bestT.cpc, bestT.spl, bestT.lanes);
  if (rc) return rc;
  rc = batch_snapshot(bt, true);
  if (rc) return rc;
  bt->steps_done = steps0;
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return MCGPU_OK;
}
