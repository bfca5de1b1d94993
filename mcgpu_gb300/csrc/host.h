// host.h -- host-side internals shared by the C-ABI translation units
// (abi.cu: boxes and batches; server.cu: the serving loop): the context,
// error reporting, the host and device pool layouts and the pool helpers.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <memory>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "device.cuh"

namespace mcgpu {

// ---- kernels (kernels.cu, npt.cu) ----
__global__ void k_refresh_mirrors(Pool P, const int* mol_chain, int m_begin, int m_end);
__global__ void k_blend_rows(Pool P, int n_atom);
__global__ void k_change_molecule(Pool P, int chain, int mol, Proposal prop, SmemShape shape);
__global__ void k_rollback(Pool P, int chain, int mol);
__global__ void k_chain_sums(Pool P, const double* emol, double* out);
__global__ void k_set_energy(Pool P, const double* e);
__global__ void k_chain_steps(Pool P, int n_steps, unsigned* queue, const int* order, int n_tasks,
                              int gwarps, SmemShape shape, mcgpu_trace* trace, int trace_off,
                              int trace_stride, int lanes_cap);
__global__ void k_chain_steps_wide(Pool P, int n_steps, unsigned* queue, const int* order,
                                   int n_tasks, int gwarps, SmemShape shape, mcgpu_trace* trace,
                                   int trace_off, int trace_stride, int lanes_cap);
__global__ void k_chain_init(Pool P, const int* mol_chain, int m_begin, int m_end);
__global__ void k_chain_energy1(Pool P, int c, const double* emol);
__global__ void k_nl_config(Pool P, const NlCfg* cfg);
cudaError_t launch_nl_rebuild(Pool P, const int* mol_chain, int n_mol, int max_cells,
                              cudaStream_t st);
__global__ void k_chain_export(Pool P, const int* mol_chain, const int* atom_mol, int a_begin,
                               int a_end);
cudaError_t launch_mol_energy(bool f64, int grid, int threads, SmemShape sh, cudaStream_t st,
                              Pool P, int chain, int curr, int start, double* partials,
                              unsigned* counter, double* out, long long* pairs = nullptr);
cudaError_t launch_move_energies(bool f64, int grid, int threads, SmemShape sh, cudaStream_t st,
                                 Pool P, int chain, int mol, Proposal prop, double* partials,
                                 unsigned* counter, double* out, long long* pairs = nullptr);
cudaError_t launch_mol_pair_sums(bool f64, int grid, int threads, SmemShape sh, cudaStream_t st,
                                 Pool P, const int* mol_chain, int m_begin, double* emol,
                                 long long* pairs);
// One volume phase of the chains in act (all when act has no ranges) on
// stream st: proposals, cell grids, FP32 / FP64 totals, decisions, the
// double-float and FP64 re-takes; vlist holds 3 * (chains) + 3 ints.
cudaError_t launch_volume_phase(Pool P, const int* mol_chain, int n_mol_total, VolMove* vm,
                                double2* emol2, double2* eabs2, double2* esum, double2* esum_abs,
                                int* vlist, mcgpu_vol_trace* trace, int trace_slot,
                                int trace_stride, cudaStream_t st, MolRanges act, bool has64,
                                bool has32);
cudaError_t launch_chain_energy(Pool P, const int* mol_chain, int n_mol_total, VolMove* vm,
                                double2* emol2, double2* eabs2, double2* esum, double2* esum_abs,
                                cudaStream_t st, MolRanges act, bool f64);

}  // namespace mcgpu

struct mcgpu_ctx {
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;   // stream every launch goes to
  cudaStream_t own = nullptr;      // the context's own stream
  std::string err;
};

// Records an error for the context (and the process) and returns code.
int set_err(mcgpu_ctx* ctx, int code, const char* fmt, ...);

#define CK(ctx, call)                                                                  \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess)                                                             \
      return set_err((ctx), MCGPU_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

namespace mcgpu {

template <class T>
T* dalloc(size_t n, cudaError_t* e) {
  T* p = nullptr;
  cudaError_t r = cudaMalloc((void**)&p, sizeof(T) * std::max<size_t>(n, 1));
  if (r != cudaSuccess && *e == cudaSuccess) *e = r;
  return p;
}

// Allocator whose construction without a value leaves trivial types
// uninitialised: resize() of the host rows costs no fill (the pool build
// writes every entry afterwards).
template <class T>
struct NoFillAlloc : std::allocator<T> {
  template <class U>
  struct rebind {
    using other = NoFillAlloc<U>;
  };
  NoFillAlloc() = default;
  template <class U>
  NoFillAlloc(const NoFillAlloc<U>&) noexcept {}
  template <class U>
  void construct(U* p) noexcept(std::is_nothrow_default_constructible<U>::value) {
    ::new ((void*)p) U;
  }
  template <class U, class... A>
  void construct(U* p, A&&... a) {
    ::new ((void*)p) U(std::forward<A>(a)...);
  }
};
template <class T>
using HostRow = std::vector<T, NoFillAlloc<T>>;

struct HostPool {
  HostRow<double> x, y, z, sig, eps, q;
  HostRow<float4> aoff;
  HostRow<float2> aeq;
  HostRow<int> mstart, mlen, pidx, mol_chain, atom_mol;
  HostRow<int2> mpi;
  HostRow<float> mrad;
  HostRow<ChainHdr> hdr;
  int max_len = 0;
  // capacity for the given totals (one allocation per row instead of growth)
  void reserve(size_t atoms, size_t mols, size_t pidxs, size_t chains) {
    for (auto* v : {&x, &y, &z, &sig, &eps, &q}) v->reserve(atoms);
    aoff.reserve(atoms);
    aeq.reserve(atoms);
    atom_mol.reserve(atoms);
    for (auto* v : {&mstart, &mlen, &mol_chain}) v->reserve(mols);
    mpi.reserve(mols);
    mrad.reserve(mols);
    pidx.reserve(pidxs);
    hdr.reserve(chains);
  }
  // rows of exactly the given totals (new entries value-initialised)
  void resize(size_t atoms, size_t mols, size_t pidxs, size_t chains) {
    for (auto* v : {&x, &y, &z, &sig, &eps, &q}) v->resize(atoms);
    aoff.resize(atoms);
    aeq.resize(atoms);
    atom_mol.resize(atoms);
    for (auto* v : {&mstart, &mlen, &mol_chain}) v->resize(mols);
    mpi.resize(mols);
    mrad.resize(mols);
    pidx.resize(pidxs);
    hdr.resize(chains);
  }
};

// Validates one descriptor and appends it as chain `c` of the host pool.
int append_chain(mcgpu_ctx* ctx, HostPool& hp, const mcgpu_box_desc* d, int c,
                 unsigned long long seed, int rot_mode);
// The host pool of descs[0..n) (chain c seeded with seeds[c]), built on
// several host threads; errors as append_chain reports them chain by chain.
int build_pool(mcgpu_ctx* ctx, HostPool& hp, const mcgpu_box_desc* descs, int n,
               const uint64_t* seeds, int rot_mode);

struct DevPool {
  Pool P{};
  int n_chains = 0, n_mol = 0, n_atom = 0, n_pidx = 0, max_len = 0;
  int* mol_chain = nullptr;
  int* atom_mol = nullptr;
  double* emol = nullptr;
  long long* pairs = nullptr;
  double* esum = nullptr;
  std::vector<ChainHdr> hdr;  // host copy of the headers at upload
  std::vector<int> mstart, mlen;  // host copies (pool-absolute)
  bool nl_on = false;             // some chain keeps a Verlet list
  int nl_max_cells = 0;           // largest per-chain cell allocation

  void release() {
    void* ptrs[] = {P.x, P.y, P.z, P.sig, P.eps, P.q, P.aoff, P.aofl, P.blend, P.aeq, P.mstart,
                    P.mlen, P.mpi,
                    P.mfix, P.mrad, P.mq, P.atpl, P.pidx, P.ppos, P.hdr, P.rb, P.trace,
                    P.nl, P.nl_cnt, P.pbuild, P.mcell, P.cell_cnt, P.cell_start, P.cell_mol,
                    P.vc_cnt, P.vc_start, P.vc_mol, P.vc_of,
                    mol_chain, atom_mol, emol, pairs, esum};
    for (void* p : ptrs)
      if (p) cudaFree(p);
    P = Pool{};
    mol_chain = nullptr;
    atom_mol = nullptr;
    emol = nullptr;
    pairs = nullptr;
    esum = nullptr;
  }
};

int upload_pool(mcgpu_ctx* ctx, HostPool& hp, DevPool& dp);
SmemShape shape_for(int max_len, int nwarps, int cache_n = 0);

// Largest chain whose primary screen positions a group caches in shared
// memory (16 bytes per molecule).
constexpr int kCacheMax = 4096;

int pool_cache_n(const DevPool& dp);
int pool_chain_init(mcgpu_ctx* ctx, DevPool& dp, cudaStream_t st);
int pool_chain_export(mcgpu_ctx* ctx, DevPool& dp, cudaStream_t st);
int pool_system_energy(mcgpu_ctx* ctx, DevPool& dp, bool f64, cudaStream_t st);
// Verlet lists with the given skin for every chain (skin <= 0: off).
int pool_set_verlet(mcgpu_ctx* ctx, DevPool& dp, double skin, cudaStream_t st);
// Rebuilds the stale lists (no-op launches when none is stale).
int pool_nl_rebuild(mcgpu_ctx* ctx, DevPool& dp, cudaStream_t st);

// ---- windowed chain kernel (window.cu) ----------------------------------------
// Shared memory the windowed kernel may use per CTA.
constexpr int kWindowSmemMax = 220 * 1024;
// Dynamic shared memory of one CTA of a K-step window for group shape sh.
int window_smem_bytes(const SmemShape& sh, int K);
// Enables the kernel's shared memory (once per context).
cudaError_t window_init();
// Clusters of K CTAs (threads, smem bytes each) that fit on the device at
// once (0 if none).
int window_max_clusters(int K, int threads, int smem);
// n_clusters clusters of K CTAs of `threads` threads, chain tasks order[0
// .. n_tasks) advanced n_steps steps each in windows of K steps.
cudaError_t launch_chain_window(int K, int n_clusters, int threads, int smem, cudaStream_t st,
                                const Pool& P, int n_steps, const int* order, int n_tasks,
                                SmemShape sh, mcgpu_trace* trace, int trace_off, int trace_stride,
                                int lanes_cap);

}  // namespace mcgpu
