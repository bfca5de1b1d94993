// nlist.cu -- Verlet neighbour lists of device-resident chains, built on the
// GPU from a cell list.
//
// A chain's list of molecule i holds every molecule j whose anchor (first
// primary atom) was within r_list = rc + skin + 2 prad of i's anchor at the
// build, prad the largest primary-to-anchor distance of the chain.  While
// every primary of every molecule stays within skin/2 of its position at
// the build, any molecule pair with a primary pair inside rc is in the list,
// so the chain kernel screens the list instead of all molecules and finds
// the same in-range set (the screen itself is unchanged).  The kernel checks
// the trial placement against skin/2 (full scan for that step if it is
// farther) and marks the list stale when such a placement is accepted; the
// rebuild below runs between launches for stale chains only.
//
// Cells: ncell[k] = floor(L_k / r_list) per edge (at least 1, at most the
// chain's allocated cells); molecule m is in cell floor(A_k * ncell[k] /
// 2^32) of its fixed-point anchor A, exact and wrap-free.  Each cell's
// members are sorted by index and each list is written cell by cell in a
// fixed stencil order, so the lists (and the pair summation order that
// follows them) are deterministic.
#include "chain.cuh"

namespace mcgpu {

__device__ __forceinline__ bool nl_rebuilding(const ChainHdr& H) { return H.nl_on && !H.nl_valid; }

// Cell grid of every stale chain from its current box; zero the counters.
__global__ void k_nl_reset(Pool P) {
  ChainHdr& H = P.hdr[blockIdx.x];
  if (!nl_rebuilding(H)) return;
  __shared__ int nc[3];
  if (threadIdx.x == 0) {
    for (int k = 0; k < 3; k++) nc[k] = max(1, (int)floor(H.L[k] / (double)H.nl_rlist));
    // fewer, larger cells if the grid outgrew its allocation (box growth)
    while (nc[0] * nc[1] * nc[2] > H.cell_cap) {
      int kmax = 0;
      for (int k = 1; k < 3; k++)
        if (nc[k] > nc[kmax]) kmax = k;
      nc[kmax]--;
    }
    for (int k = 0; k < 3; k++) H.ncell[k] = nc[k];
  }
  __syncthreads();
  const int n = nc[0] * nc[1] * nc[2];
  for (int i = threadIdx.x; i < n; i += blockDim.x) P.cell_cnt[H.cell0 + i] = 0;
}

__device__ __forceinline__ int cell_of(unsigned a, int n) {
  return (int)(((unsigned long long)a * (unsigned)n) >> 32);
}

__global__ void k_nl_count(Pool P, const int* mol_chain, int n_mol) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n_mol) return;
  const ChainHdr& H = P.hdr[mol_chain[m]];
  if (!nl_rebuilding(H)) return;
  const uint4 A = P.mfix[m];
  const int cx = cell_of(A.x, H.ncell[0]), cy = cell_of(A.y, H.ncell[1]), cz = cell_of(A.z, H.ncell[2]);
  const int cell = H.cell0 + (cx * H.ncell[1] + cy) * H.ncell[2] + cz;
  P.mcell[m] = cell;
  atomicAdd(&P.cell_cnt[cell], 1);
}

// Exclusive scan of a stale chain's cell counts into cell_start (pool
// positions from the chain's first molecule); counters reset for the fill.
__global__ void k_nl_scan(Pool P) {
  const ChainHdr& H = P.hdr[blockIdx.x];
  if (!nl_rebuilding(H) || threadIdx.x != 0) return;
  const int n = H.ncell[0] * H.ncell[1] * H.ncell[2];
  int run = H.mol0;
  for (int i = 0; i < n; i++) {
    const int c = H.cell0 + i;
    P.cell_start[c] = run;
    run += P.cell_cnt[c];
    P.cell_cnt[c] = 0;
  }
}

__global__ void k_nl_scatter(Pool P, const int* mol_chain, int n_mol) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n_mol) return;
  const ChainHdr& H = P.hdr[mol_chain[m]];
  if (!nl_rebuilding(H)) return;
  const int cell = P.mcell[m];
  const int pos = atomicAdd(&P.cell_cnt[cell], 1);
  P.cell_mol[P.cell_start[cell] + pos] = m;
}

// Sorts each cell's members by index (insertion sort; cells hold tens of
// molecules).  One thread per cell; blockIdx.y is the chain.
__global__ void k_nl_sort(Pool P) {
  const ChainHdr& H = P.hdr[blockIdx.y];
  if (!nl_rebuilding(H)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= H.ncell[0] * H.ncell[1] * H.ncell[2]) return;
  const int c = H.cell0 + i;
  int* v = P.cell_mol + P.cell_start[c];
  const int n = P.cell_cnt[c];
  for (int a = 1; a < n; a++) {
    const int key = v[a];
    int b = a - 1;
    while (b >= 0 && v[b] > key) {
      v[b + 1] = v[b];
      b--;
    }
    v[b + 1] = key;
  }
}

// Cells of the stencil along one edge: c-1, c, c+1 (periodic) when the edge
// has at least 3 cells, else every cell once.
__device__ __forceinline__ int stencil(int c, int n, int* out) {
  if (n >= 3) {
    out[0] = (c + n - 1) % n;
    out[1] = c;
    out[2] = (c + 1) % n;
    return 3;
  }
  for (int k = 0; k < n; k++) out[k] = k;
  return n;
}

// One warp per molecule of a stale chain: its list from the stencil cells,
// appended in cell order and member order; the build positions of its
// primaries.
__global__ void k_nl_build(Pool P, const int* mol_chain, int n_mol) {
  const int m = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (m >= n_mol) return;
  ChainHdr& H = P.hdr[mol_chain[m]];
  if (!nl_rebuilding(H)) return;
  const int2 pi = P.mpi[m];
  for (int k = lane; k < pi.y; k += 32) P.pbuild[pi.x + k] = P.ppos[pi.x + k];
  const float4 am = P.ppos[pi.x];
  const int local = P.mcell[m] - H.cell0;
  const int n1 = H.ncell[1], n2 = H.ncell[2];
  const int cz = local % n2, cy = (local / n2) % n1, cx = local / (n1 * n2);
  int sx[3], sy[3], sz[3];
  const int nx = stencil(cx, H.ncell[0], sx), ny = stencil(cy, n1, sy), nz = stencil(cz, n2, sz);
  int* out = P.nl + (size_t)m * P.nl_stride;
  int cnt = 0;
  bool over = false;
  const unsigned lt = lanemask_lt();
  for (int a = 0; a < nx; a++)
    for (int b = 0; b < ny; b++)
      for (int c = 0; c < nz; c++) {
        const int cell = H.cell0 + (sx[a] * n1 + sy[b]) * n2 + sz[c];
        const int s0 = P.cell_start[cell], n = P.cell_cnt[cell];
        for (int base = 0; base < n; base += 32) {
          const int t = base + lane;
          bool in = false;
          int j = -1;
          if (t < n) {
            j = P.cell_mol[s0 + t];
            if (j != m) in = r2_screen(am, P.ppos[P.mpi[j].x], H) <= H.nl_r2;
          }
          const unsigned bal = __ballot_sync(~0u, in);
          const int at = cnt + __popc(bal & lt);
          if (in) {
            if (at < P.nl_stride) out[at] = j;
            else over = true;
          }
          cnt += __popc(bal);
        }
      }
  over = __any_sync(~0u, over);
  if (lane == 0) {
    P.nl_cnt[m] = min(cnt, P.nl_stride);
    if (over) atomicAdd(&H.nl_overflow, 1);
  }
}

// Marks rebuilt lists valid (an overflowing chain drops its list: full
// scans stay exact).
__global__ void k_nl_finish(Pool P) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= P.n_chains) return;
  ChainHdr& H = P.hdr[c];
  if (!nl_rebuilding(H)) return;
  if (H.nl_overflow) {
    H.nl_on = 0;
    return;
  }
  H.nl_valid = 1;
  H.nl_builds++;
}

// Per-chain list configuration (host-computed), applied to the headers.
__global__ void k_nl_config(Pool P, const NlCfg* cfg) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= P.n_chains) return;
  ChainHdr& H = P.hdr[c];
  const NlCfg f = cfg[c];
  H.nl_on = f.on;
  H.nl_valid = 0;
  H.nl_overflow = 0;
  H.cell0 = f.cell0;
  H.cell_cap = f.cell_cap;
  H.nl_r2 = f.r2;
  H.nl_half2 = f.half2;
  H.nl_rlist = f.rlist;
}

cudaError_t launch_nl_rebuild(Pool P, const int* mol_chain, int n_mol, int max_cells,
                              cudaStream_t st) {
  const int nc = P.n_chains;
  k_nl_reset<<<nc, 256, 0, st>>>(P);
  k_nl_count<<<(n_mol + 255) / 256, 256, 0, st>>>(P, mol_chain, n_mol);
  k_nl_scan<<<nc, 32, 0, st>>>(P);
  k_nl_scatter<<<(n_mol + 255) / 256, 256, 0, st>>>(P, mol_chain, n_mol);
  k_nl_sort<<<dim3((max_cells + 127) / 128, nc), 128, 0, st>>>(P);
  k_nl_build<<<(n_mol + 7) / 8, 256, 0, st>>>(P, mol_chain, n_mol);
  k_nl_finish<<<(nc + 127) / 128, 128, 0, st>>>(P);
  return cudaGetLastError();
}

}  // namespace mcgpu
