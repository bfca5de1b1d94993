// static_energy.cu -- mcgpu_system_energy_static: the FP64 system energy
// (SimulationStep::calcSystemEnergy's sum, the reference's pair arithmetic)
// over SimBox rows that the CALLER already holds in device memory, without
// allocating anything.
//
// Who needs it: programs that cannot call cudaMalloc for this library --
// an OpenACC or OpenMP-offload build that keeps its SimBox rows in its own
// device data region (as MCGPU's -p build does through acc_copyin), or an
// application whose device memory is owned by another allocator (a
// framework's caching allocator, a fixed arena of a long-running service)
// and forbids allocations from third-party code.  They pass device pointers
// to their rows and to one output double; the per-molecule partial energies
// live in a fixed file-scope device array instead of a cudaMalloc'd buffer.
//
// Limits and sharing: at most kStaticMaxMol molecules per call (larger boxes
// are rejected with MCGPU_ERR_UNSUPPORTED).  Every GPU that loads the
// library holds the array (kStaticMaxMol doubles, 256 KiB) until the process
// exits.  All calls on a device share it and it keeps the last call's
// contents; each entry a call reads was written earlier in that same call,
// so nothing needs clearing, but calls that overlap on the GPU (different
// streams, no ordering) race on it.  The first call on each device looks up
// the array's device address (cudaGetSymbolAddress) with that device
// current and caches it; make that first call before any stream capture.
// The cache is keyed on the current context's id: after a device reset or a
// new primary context the next call looks the address up again (that call
// is then a first call, with the same rule on capture).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>

#include "../../include/mcgpu_gb300.h"
#include "static_scratch_cache.h"

namespace mcgpu {
void note_process_error(const char* msg);  // abi.cu: text for mcgpu_last_error(NULL)
}

namespace {
constexpr int kStaticMaxMol = 32768;
constexpr int kMaxDevices = 64;
}  // namespace

// The scratch: E(m, j > m) for every molecule m of the box, one copy per
// device, never cleared (every entry a call reads, it wrote first).
static __device__ __align__(256) double g_static_emol[kStaticMaxMol];

namespace {

struct Rows {
  const double *x, *y, *z, *sig, *eps, *q;
  const int *mstart, *mlen, *mps, *mpc, *pidx;
  int n_mol, n_atom, n_pidx;
  double L[3], cutoff;
};

// SimCalcs::makePeriodic (SimulationStep.cpp:377-385).
__device__ __forceinline__ double periodic(double x, double L) {
  if (x < -0.5 * L) x = __dadd_rn(x, L);
  if (x > 0.5 * L) x = __dadd_rn(x, -L);
  return x;
}

// SimCalcs::calcAtomDistSquared (SimulationStep.cpp:332-342), a2 - a1.
__device__ __forceinline__ double dist2(const Rows& r, int a1, int a2) {
  const double dx = periodic(r.x[a2] - r.x[a1], r.L[0]);
  const double dy = periodic(r.y[a2] - r.y[a1], r.L[1]);
  const double dz = periodic(r.z[a2] - r.z[a1], r.L[2]);
  return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

// Row ranges of molecule m inside the arrays.  A molecule without primary
// indexes (pc == 0) is valid: moleculesInRange is false for it
// (SimulationStep.cpp:317-330), so it contributes nothing.
__device__ __forceinline__ bool valid_mol(const Rows& r, int m) {
  const int s = r.mstart[m], n = r.mlen[m], ps = r.mps[m], pc = r.mpc[m];
  return s >= 0 && n >= 1 && s + n <= r.n_atom && ps >= 0 && pc >= 0 && ps + pc <= r.n_pidx;
}

// E(m, j > m) per CTA m: threads stride over candidates j; the reference's
// primary-pair cutoff (SimulationStep.cpp:317-330) and FP64 pair terms
// (BruteForceStep.cpp:48-79, SimulationStep.cpp:344-375).  A molecule with
// out-of-range rows makes the partial NaN instead of reading past them.
__global__ void k_static_pair_sums(Rows r, double* emol) {
  const int m = blockIdx.x;
  __shared__ double red[256];
  double acc = 0.0;
  bool bad = !valid_mol(r, m);
  if (!bad) {
    const int s1 = r.mstart[m], e1 = s1 + r.mlen[m];
    const int p1s = r.mps[m], p1e = p1s + r.mpc[m];
    for (int j = m + 1 + (int)threadIdx.x; j < r.n_mol; j += blockDim.x) {
      if (!valid_mol(r, j)) {
        bad = true;
        continue;
      }
      bool in = false;
      for (int p1 = p1s; p1 < p1e && !in; p1++)
        for (int p2 = r.mps[j]; p2 < r.mps[j] + r.mpc[j] && !in; p2++) {
          const int a1 = r.pidx[p1], a2 = r.pidx[p2];
          if (a1 < 0 || a1 >= r.n_atom || a2 < 0 || a2 >= r.n_atom) {
            bad = true;
            break;
          }
          in = dist2(r, a1, a2) <= __dmul_rn(r.cutoff, r.cutoff);
        }
      if (!in) continue;
      const int s2 = r.mstart[j], e2 = s2 + r.mlen[j];
      double e = 0.0;
      for (int i = s1; i < e1; i++)
        for (int k = s2; k < e2; k++) {
          const double si = r.sig[i], sk = r.sig[k], ei = r.eps[i], ek = r.eps[k];
          if (!(si >= 0 && sk >= 0 && ei >= 0 && ek >= 0)) continue;
          const double r2 = dist2(r, i, k);
          if (r2 == 0.0) continue;
          const double ss = si * sk, ee = ei * ek;
          const double sigma = sqrt(ss >= 0 ? ss : -ss);
          const double eps = sqrt(ee >= 0 ? ee : -ee);
          const double s2r2 = (sigma * sigma) / r2;
          const double s6 = s2r2 * s2r2 * s2r2;
          e += 4.0 * eps * (s6 * s6 - s6);
          e += (r.q[i] * r.q[k] * 332.06) / sqrt(r2);
        }
      acc += e;
    }
  }
  red[threadIdx.x] = bad ? __longlong_as_double(0x7ff8000000000000LL) : acc;
  __syncthreads();
  for (int off = blockDim.x >> 1; off > 0; off >>= 1) {
    if ((int)threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0) emol[m] = red[0];
}

// Ordered sum of the partials into *out (thread t adds every blockDim-th
// term from t, then a fixed tree).
__global__ void k_static_sum(const double* emol, int n, double* out) {
  __shared__ double red[256];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += emol[i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int off = blockDim.x >> 1; off > 0; off >>= 1) {
    if ((int)threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

mcgpu::ScratchAddressCache<kMaxDevices> g_emol_cache;  // device address of the scratch

int fail(int code, const char* msg) {
  mcgpu::note_process_error(msg);
  return code;
}

// Id of the calling thread's current context (0 if none or unknown), through
// the driver's cuCtxGetCurrent / cuCtxGetId fetched from the runtime (no link
// against the driver library).
typedef int (*PfnCtxGetCurrent)(void**);
typedef int (*PfnCtxGetId)(void*, unsigned long long*);

unsigned long long current_context_id() {
  static std::once_flag once;
  static PfnCtxGetCurrent get_current = nullptr;
  static PfnCtxGetId get_id = nullptr;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = (PfnCtxGetCurrent)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = (PfnCtxGetId)f;
  });
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx) return 0;
  if (get_id(ctx, &id) != 0) return 0;
  return id;
}

}  // namespace

extern "C" int mcgpu_system_energy_static(const mcgpu_box_desc* rows, double* out, void* stream) {
  if (!rows || !out) return fail(MCGPU_ERR_INVALID, "null argument");
  if (rows->n_mol <= 0 || rows->n_atom <= 0 || rows->n_pidx <= 0)
    return fail(MCGPU_ERR_INVALID, "empty box");
  if (rows->n_mol > kStaticMaxMol)
    return fail(MCGPU_ERR_UNSUPPORTED,
                "mcgpu_system_energy_static: more than 32768 molecules (its fixed scratch holds "
                "one partial per molecule); use mcgpu_system_energy");
  if (!rows->x || !rows->y || !rows->z || !rows->sigma || !rows->epsilon || !rows->charge ||
      !rows->mol_start || !rows->mol_len || !rows->mol_pidx_start || !rows->mol_pidx_count ||
      !rows->pidx)
    return fail(MCGPU_ERR_INVALID, "null row pointer");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail(MCGPU_ERR_CUDA, "no current CUDA device");
  double* emol = (double*)g_emol_cache.get(
      dev, current_context_id(),
      [](void** p) { return cudaGetSymbolAddress(p, g_static_emol) == cudaSuccess; },
      [] { return current_context_id(); });
  if (!emol) return fail(MCGPU_ERR_CUDA, "cudaGetSymbolAddress of the static scratch failed");
  Rows r;
  r.x = rows->x; r.y = rows->y; r.z = rows->z;
  r.sig = rows->sigma; r.eps = rows->epsilon; r.q = rows->charge;
  r.mstart = rows->mol_start; r.mlen = rows->mol_len;
  r.mps = rows->mol_pidx_start; r.mpc = rows->mol_pidx_count; r.pidx = rows->pidx;
  r.n_mol = rows->n_mol; r.n_atom = rows->n_atom; r.n_pidx = rows->n_pidx;
  for (int k = 0; k < 3; k++) r.L[k] = rows->size[k];
  r.cutoff = rows->cutoff;
  cudaStream_t st = (cudaStream_t)stream;
  // An error the caller's own code left pending stays the caller's: it is
  // neither cleared nor reported as this call's.
  const cudaError_t prior = cudaPeekAtLastError();
  auto launch_error = [prior]() {
    const cudaError_t e = prior == cudaSuccess ? cudaGetLastError() : cudaPeekAtLastError();
    return e == prior ? cudaSuccess : e;
  };
  k_static_pair_sums<<<r.n_mol, 256, 0, st>>>(r, emol);
  cudaError_t e = launch_error();
  if (e == cudaSuccess) {
    k_static_sum<<<1, 256, 0, st>>>(emol, r.n_mol, out);
    e = launch_error();
  }
  if (e != cudaSuccess) {
    static thread_local char msg[256];
    snprintf(msg, sizeof(msg), "mcgpu_system_energy_static: launch failed: %s",
             cudaGetErrorString(e));
    return fail(MCGPU_ERR_CUDA, msg);
  }
  return MCGPU_OK;
}
