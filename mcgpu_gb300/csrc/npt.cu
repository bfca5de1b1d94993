// npt.cu -- isobaric (NPT) volume moves of device-resident chains.
//
// A volume move of a chain whose step count is a multiple of its interval:
//   ln V' = ln V + dlnv,  dlnv uniform in +-max_dlnv (Philox block 3 of the
//   step's counter), every edge scaled by s = exp(dlnv / 3);
//   each molecule's centre (its first primary atom, the chain state's
//   anchor) scales about the origin, c' = s c, its geometry stays rigid.  In
//   the chain state the anchor is a fixed-point fraction of the edge, so the
//   scaling is the change of L alone;
//   accepted when exp(-(dU + P dV)/kT + (N + 1) dlnv) >= u (u from the same
//   Philox block), with U(V) and U(V') full FP64 system energies (the
//   reference's pair arithmetic, SimulationStep.cpp:40-71, :317-375) of the
//   chain state at both volumes.
// The reference's own NPT path (Ensemble.cpp:9-23, SimulationStep.cpp:476-518)
// applies a fixed factor 1.1 and no pressure units; this is the standard
// isobaric ln V move instead.  The running energy is replaced by the FP64
// total of the volume the chain keeps (a drift reset every interval).
//
// With vol_mixed U(V) is the running energy and U(V') comes from FP32 pair
// terms summed in double-float (k_vol_pair_sums32); the decision is taken on
// them unless the criterion's argument lies within their error bound of
// ln u.  Those chains alone are re-evaluated -- U(V') in double-float, then
// both totals in double-float, then both in FP64, each tier only for what the
// last left too close to call -- so the decisions are the FP64 ones.
//
// Kernels (one volume phase, launched between step launches):
//   k_vol_propose      per chain: due?, draw, L'
//   k_vol_pair_sums    per molecule: E(m, j>m) at V and V' (FP64 pairs)
//   k_vol_pair_sums32  the same with FP32 pairs (vol_mixed chains)
//   k_vol_sums         per chain: ordered sums
//   k_vol_decide       per chain: criterion (or the FP64 re-take mark), new
//                      box, energy
//   k_vol_refresh      per molecule of an accepting chain: screen positions
#include "chain.cuh"

namespace mcgpu {

// exp(x) for |x| <= 0.034 by its Taylor series to x^6 (Horner, every
// operation rounded once): relative truncation error below 1e-14.  The
// oracle evaluates the same expression, so the scaled box is bit-identical.
__device__ __forceinline__ double exp_small(double x) {
  double p = 1.0 / 720.0;
  p = __dadd_rn(__dmul_rn(p, x), 1.0 / 120.0);
  p = __dadd_rn(__dmul_rn(p, x), 1.0 / 24.0);
  p = __dadd_rn(__dmul_rn(p, x), 1.0 / 6.0);
  p = __dadd_rn(__dmul_rn(p, x), 0.5);
  p = __dadd_rn(__dmul_rn(p, x), 1.0);
  p = __dadd_rn(__dmul_rn(p, x), 1.0);
  return p;
}

// Chain of work item i: i itself, or the i-th active slot.
__device__ __forceinline__ int range_chain(const MolRanges& R, int i) {
  return R.act_slot ? R.act_slot[i] : i;
}

__device__ inline void volbox_set(VolBox& B, const double* L, double rc) {
  double Lmax = 0;
  for (int k = 0; k < 3; k++) {
    B.L[k] = L[k];
    B.Lf[k] = (float)L[k];
    B.fxs[k] = (float)(L[k] / 4294967296.0);
    B.fxs_lo[k] = (float)(L[k] / 4294967296.0 - (double)B.fxs[k]);
    Lmax = fmax(Lmax, L[k]);
  }
  const double band = screen_band(rc, Lmax);
  B.cut2_lo = (float)(rc * rc - band);
  B.cut2_hi = (float)(rc * rc + band);
}

__device__ __forceinline__ float vol_reach(const ChainHdr& H) {
  return (float)(H.cutoff + 2.0 * (double)H.prad + 1e-2);
}

__global__ void k_vol_propose(Pool P, VolMove* vm, MolRanges R, int n_items) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_items) return;
  const int c = range_chain(R, i);
  const ChainHdr& H = P.hdr[c];
  VolMove v;
  v.state = 0;
  v.fp64 = 0;
  v.dlnv = 0.0;
  v.u = 0.0;
  for (int k = 0; k < 3; k++) v.L[k] = H.L[k];
  if (H.vol_interval > 0 && H.step > 0 && H.step % (unsigned long long)H.vol_interval == 0 &&
      (long long)H.step > H.vol_step && H.error == 0) {
    const uint2 key = make_uint2((unsigned)H.seed, (unsigned)(H.seed >> 32));
    const uint4 r = philox4x32_10(
        make_uint4((unsigned)H.step, (unsigned)(H.step >> 32), (unsigned)H.chain_id, 3u), key);
    v.dlnv = __dadd_rn(__dmul_rn(2.0 * H.max_dlnv, u01(r.x)), -H.max_dlnv);
    v.u = u01(r.y);
    const double s = exp_small(v.dlnv / 3.0);
    double Lmin = 1e300;
    for (int k = 0; k < 3; k++) {
      v.L[k] = __dmul_rn(H.L[k], s);
      Lmin = fmin(Lmin, v.L[k]);
    }
    volbox_set(v.box[0], H.L, H.cutoff);
    volbox_set(v.box[1], v.L, H.cutoff);
    v.reach = vol_reach(H);
    v.sf = (float)(v.L[0] / H.L[0]);
    // molecules must stay within a quarter of an edge (the chain state's
    // anchor-image rule); the cutoff may exceed half an edge, as in the
    // reference's single-image minimum convention
    v.state = ((double)H.rad_max >= 0.25 * Lmin) ? 2 : 1;
  }
  vm[c] = v;
}

// FP64 position of a chain atom at box edge L (anchor fraction scaled).
__device__ __forceinline__ double3 pos_at(uint4 A, float4 o, const double* L) {
  return make_double3(chain_coord(A.x, o.x, L[0]), chain_coord(A.y, o.y, L[1]),
                      chain_coord(A.z, o.z, L[2]));
}

__device__ __forceinline__ double dist2_at(double3 a, double3 b, const double* L) {
  const double dx = make_periodic(b.x - a.x, L[0]);
  const double dy = make_periodic(b.y - a.y, L[1]);
  const double dz = make_periodic(b.z - a.z, L[2]);
  return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

constexpr int kVolThreads = 128;
// CTAs of the grid-strided re-take kernels (a few per SM)
constexpr int kVolListGrid = 152 * 4;

// Pool molecule of work item b: m_begin + b, or the b-th molecule of the
// active ranges (binary search over their prefix sums).
__device__ __forceinline__ int range_mol(const MolRanges& R, int m_begin, int b) {
  if (!R.act_pref) return m_begin + b;
  int lo = 0, hi = R.n_act - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (R.act_pref[mid] <= b) lo = mid; else hi = mid - 1;
  }
  return R.act_m0[lo] + (b - R.act_pref[lo]);
}

// ---- cell grid of a volume move ------------------------------------------
// Cells at least r = (rc + 2 prad + 0.01) / min(1, s) wide, so every pair
// with an anchor distance within reach at V or V' lies in neighbouring
// cells; cell c of a chain is pool entry mol0 + c (at most n_mol cells).


__global__ void k_vc_grid(Pool P, const VolMove* vm, MolRanges R, int n_items) {
  const int i = blockIdx.x;
  if (i >= n_items) return;
  const int c = range_chain(R, i);
  if (vm[c].state != 1) return;
  ChainHdr& H = P.hdr[c];
  __shared__ int nc[3];
  if (threadIdx.x == 0) {
    const double s = vm[c].L[0] / H.L[0];
    const double edge = (double)vol_reach(H) / fmin(1.0, s) * (1.0 + 1e-6);
    for (int k = 0; k < 3; k++) nc[k] = max(1, (int)floor(H.L[k] / edge));
    while ((long long)nc[0] * nc[1] * nc[2] > H.n_mol) {
      int kmax = 0;
      for (int k = 1; k < 3; k++)
        if (nc[k] > nc[kmax]) kmax = k;
      nc[kmax]--;
    }
    for (int k = 0; k < 3; k++) H.vncell[k] = nc[k];
  }
  __syncthreads();
  const int n = nc[0] * nc[1] * nc[2];
  for (int k = threadIdx.x; k < n; k += blockDim.x) P.vc_cnt[H.mol0 + k] = 0;
}

__device__ __forceinline__ int vcell_of(unsigned a, int n) {
  return (int)(((unsigned long long)a * (unsigned)n) >> 32);
}

__global__ void k_vc_count(Pool P, const int* mol_chain, const VolMove* vm, MolRanges R,
                           int n_items) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n_items) return;
  const int m = range_mol(R, 0, b);
  const int c = mol_chain[m];
  if (vm[c].state != 1) return;
  const ChainHdr& H = P.hdr[c];
  const uint4 A = P.mfix[m];
  const int cx = vcell_of(A.x, H.vncell[0]), cy = vcell_of(A.y, H.vncell[1]);
  const int cz = vcell_of(A.z, H.vncell[2]);
  const int cell = H.mol0 + (cx * H.vncell[1] + cy) * H.vncell[2] + cz;
  P.vc_of[m] = cell;
  atomicAdd(&P.vc_cnt[cell], 1);
}

// Exclusive scan of a chain's cell counts into vc_start (one block of 256
// threads: contiguous runs per thread, then a scan of the run totals);
// the counters are reset for the scatter.
__global__ void k_vc_scan(Pool P, const VolMove* vm, MolRanges R, int n_items) {
  __shared__ int tot[256];
  const int i = blockIdx.x;
  if (i >= n_items) return;
  const int c = range_chain(R, i);
  if (vm[c].state != 1) return;
  const ChainHdr& H = P.hdr[c];
  const int n = H.vncell[0] * H.vncell[1] * H.vncell[2];
  const int per = (n + blockDim.x - 1) / blockDim.x;
  const int k0 = threadIdx.x * per, k1 = min(n, k0 + per);
  int sum = 0;
  for (int k = k0; k < k1; k++) sum += P.vc_cnt[H.mol0 + k];
  tot[threadIdx.x] = sum;
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int t = 0; t < (int)blockDim.x; t++) {
      const int v = tot[t];
      tot[t] = run;
      run += v;
    }
  }
  __syncthreads();
  int run = H.mol0 + tot[threadIdx.x];
  for (int k = k0; k < k1; k++) {
    P.vc_start[H.mol0 + k] = run;
    run += P.vc_cnt[H.mol0 + k];
    P.vc_cnt[H.mol0 + k] = 0;
  }
}

__global__ void k_vc_scatter(Pool P, const int* mol_chain, const VolMove* vm, MolRanges R,
                             int n_items) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n_items) return;
  const int m = range_mol(R, 0, b);
  if (vm[mol_chain[m]].state != 1) return;
  const int cell = P.vc_of[m];
  const int pos = atomicAdd(&P.vc_cnt[cell], 1);
  P.vc_mol[P.vc_start[cell] + pos] = m;
}

// Sorts each cell's members by index (deterministic candidate order); the
// work item of molecule mol0 + k sorts cell k, one warp per work item
// (blocks of kVcSortWarps warps): the members are read into shared memory
// and each is written at its rank (the number of smaller members: the
// indexes are distinct).  A cell of more than kVcSortMax members (a box of
// fewer than three cells per edge) is sorted by lane 0 in place.
constexpr int kVcSortWarps = 8;
constexpr int kVcSortMax = 384;

__global__ void __launch_bounds__(32 * kVcSortWarps) k_vc_sort(Pool P, const int* mol_chain,
                                                               const VolMove* vm, MolRanges R,
                                                               int n_items) {
  __shared__ int buf[kVcSortWarps][kVcSortMax];
  const int wi = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int b = blockIdx.x * kVcSortWarps + wi;
  if (b >= n_items) return;
  const int m = range_mol(R, 0, b);
  const int c = mol_chain[m];
  if (vm[c].state != 1) return;
  const ChainHdr& H = P.hdr[c];
  if (m - H.mol0 >= H.vncell[0] * H.vncell[1] * H.vncell[2]) return;
  int* v = P.vc_mol + P.vc_start[m];
  const int n = P.vc_cnt[m];
  if (n <= kVcSortMax) {
    int* sb = buf[wi];
    for (int i = lane; i < n; i += 32) sb[i] = v[i];
    __syncwarp();
    for (int i = lane; i < n; i += 32) {
      const int key = sb[i];
      int rank = 0;
      for (int k = 0; k < n; k++) rank += sb[k] < key;
      v[rank] = key;
    }
    return;
  }
  if (lane != 0) return;
  for (int a = 1; a < n; a++) {
    const int key = v[a];
    int k = a - 1;
    while (k >= 0 && v[k] > key) {
      v[k + 1] = v[k];
      k--;
    }
    v[k + 1] = key;
  }
}

// The cells around molecule m's (27, or every cell once along an edge of
// fewer than 3): first slot and member count of each, and prefix sums, in
// shared memory; threads then take flat candidate indices.
struct VcStencil {
  int start[27], cnt[27], pref[28];
  int n;
  int half;   // cell 0 is the molecule's own (pairs j > m), cells 1.. the
              // forward half of the neighbours (every pair): each pair once
};

// The stencil cells of molecule m's cell with their members' prefix sums.
// With at least 3 cells per edge: the own cell, then the 13 neighbours of
// the forward half (offsets after (0,0,0) in x-, y-, z-nested order) --
// each pair of molecules is met once, from the molecule whose cell comes
// first, or within a cell from the lower index.  Otherwise every cell once
// (c-1, c, c+1 per edge with at least 3 cells, else all) with pairs j > m.
// Warp 0 builds it: one cell per lane, so the counts and starts arrive in
// one round trip.
__device__ inline void vc_stencil(const Pool& P, const ChainHdr& H, int m, VcStencil& S) {
  if (threadIdx.x >= 32) return;
  const int lane = threadIdx.x;
  const int local = P.vc_of[m] - H.mol0;
  const int n0 = H.vncell[0], n1 = H.vncell[1], n2 = H.vncell[2];
  const int cz = local % n2, cy = (local / n2) % n1, cx = local / (n1 * n2);
  const bool half = n0 >= 3 && n1 >= 3 && n2 >= 3;
  const int s0 = n0 >= 3 ? 3 : n0, s1 = n1 >= 3 ? 3 : n1, s2 = n2 >= 3 ? 3 : n2;
  const int n = half ? 14 : s0 * s1 * s2;
  int start = 0, cnt = 0;
  if (lane < n) {
    int x, y, z;
    if (half) {
      const int t = lane == 0 ? 13 : 13 + lane;   // 13 is the offset (0,0,0)
      x = (cx + n0 + t / 9 - 1) % n0;
      y = (cy + n1 + (t / 3) % 3 - 1) % n1;
      z = (cz + n2 + t % 3 - 1) % n2;
    } else {
      const int a = lane / (s1 * s2), b = (lane / s2) % s1, c = lane % s2;
      x = n0 >= 3 ? (cx + n0 - 1 + a) % n0 : a;
      y = n1 >= 3 ? (cy + n1 - 1 + b) % n1 : b;
      z = n2 >= 3 ? (cz + n2 - 1 + c) % n2 : c;
    }
    const int cell = H.mol0 + (x * n1 + y) * n2 + z;
    start = P.vc_start[cell];
    cnt = P.vc_cnt[cell];
  }
  int incl = cnt;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const int v = __shfl_up_sync(~0u, incl, off);
    if (lane >= off) incl += v;
  }
  if (lane < n) {
    S.start[lane] = start;
    S.cnt[lane] = cnt;
    S.pref[lane] = incl - cnt;
  }
  if (lane == n - 1) S.pref[n] = incl;
  if (lane == 0) {
    S.n = n;
    S.half = half ? 1 : 0;
  }
}

// Whether molecule m takes candidate j found in stencil cell k.
__device__ __forceinline__ bool vc_takes(const VcStencil& S, int k, int j, int m) {
  return S.half ? (k > 0 || j > m) : j > m;
}

// Candidate t of the stencil (t < S.pref[S.n]); k is the thread's cursor
// over the cells (t only grows).
__device__ __forceinline__ int vc_candidate(const Pool& P, const VcStencil& S, int t, int& k) {
  while (S.pref[k + 1] <= t) k++;
  return P.vc_mol[S.start[k] + (t - S.pref[k])];
}


// Anchor difference b - a at box B as a double-float (fixdiff_ff's split).
__device__ __forceinline__ void vol_fixdiff(uint4 b, uint4 a, const VolBox& B, float3& hi,
                                            float3& lo) {
  const int d[3] = {(int)(b.x - a.x), (int)(b.y - a.y), (int)(b.z - a.z)};
  float h[3], l[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    // d = (d >> 9) 2^9 + (d & 511): both parts exact in FP32
    const float fh = small_i2f(d[k] >> 9) * 512.0f, fl = small_i2f(d[k] & 511);
    const float p = fh * B.fxs[k];
    const float e = fmaf(fh, B.fxs[k], -p);
    const float t = fmaf(fh, B.fxs_lo[k], fmaf(fl, B.fxs[k], e));
    h[k] = p + t;
    l[k] = t - (h[k] - p);
  }
  hi = make_float3(h[0], h[1], h[2]);
  lo = make_float3(l[0], l[1], l[2]);
}

// ---- chunked candidate screening shared by the pair kernels -------------
// A chunk of kVolChunk candidates is screened (4 per thread); the in-range
// ones are compacted per warp into shared memory in candidate order (warp
// w's segment holds its 4 x 32 candidates' hits), then every thread takes
// (neighbour, neighbour atom) items, so the pair arithmetic runs on full
// warps whatever the scatter of in-range neighbours over the candidates.
constexpr int kVolWarps = kVolThreads / 32;
constexpr int kVolChunk = 4 * kVolThreads;
constexpr int kVolSeg = kVolChunk / kVolWarps;
constexpr int kVolFShift = 28;
constexpr int kVolJMask = (1 << kVolFShift) - 1;

// In-range flags of candidate j at V (bit 0) and V' (bit 1): the FP32
// screen of every primary pair, the reference's FP64 test inside the guard
// band.  Candidates whose anchors are out of reach at both volumes are
// skipped without a test.
__device__ __forceinline__ int vol_screen(const Pool& P, const ChainHdr& H, const VolBox* vb,
                                          const float4* so, const int* spa, int npidx, uint4 Am,
                                          int j, float reach2, float sf, int w0, int nvol) {
  const uint4 Aj = P.mfix[j];
  // coarse anchor distance for the reach test (error <= 2^9 L / 2^32)
  const float3 D0 = make_float3(small_i2f((int)(Aj.x - Am.x) >> 9) * (512.0f * H.fxs[0]),
                                small_i2f((int)(Aj.y - Am.y) >> 9) * (512.0f * H.fxs[1]),
                                small_i2f((int)(Aj.z - Am.z) >> 9) * (512.0f * H.fxs[2]));
  const float d2 = fmaf(D0.x, D0.x, fmaf(D0.y, D0.y, D0.z * D0.z));
  if (d2 > reach2 && d2 * sf * sf > reach2) return 0;
  const int2 pj = P.mpi[j];
  int f = 0;
  for (int w = w0; w < w0 + nvol; w++) {
    const VolBox& B = vb[w];
    float3 Dh, Dl;
    vol_fixdiff(Aj, Am, B, Dh, Dl);
    bool in = false;
    for (int k2 = 0; k2 < pj.y && !in; k2++) {
      const float4 op = P.aoff[P.pidx[pj.x + k2]];
      for (int k1 = 0; k1 < npidx && !in; k1++) {
        const float4 oa = so[spa[k1]];
        const float dx = wrapf((Dh.x + op.x) - oa.x, B.Lf[0]);
        const float dy = wrapf((Dh.y + op.y) - oa.y, B.Lf[1]);
        const float dz = wrapf((Dh.z + op.z) - oa.z, B.Lf[2]);
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        if (r2 <= B.cut2_lo) {
          in = true;
        } else if (r2 <= B.cut2_hi) {
          in = dist2_at(pos_at(Am, oa, B.L), pos_at(Aj, op, B.L), B.L) <=
               __dmul_rn(H.cutoff, H.cutoff);
        }
      }
    }
    if (in) f |= 1 << w;
  }
  return f;
}

// Appends this lane's hit (f != 0) to its warp's segment, in lane order.
__device__ __forceinline__ void vol_append(int* ent, int* wcnt, int j, int f, int r) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (r == 0 && lane == 0) wcnt[w] = 0;
  __syncwarp();
  const unsigned bal = __ballot_sync(~0u, f != 0);
  const int base = wcnt[w];
  if (f) ent[w * kVolSeg + base + __popc(bal & lanemask_lt())] = j | (f << kVolFShift);
  __syncwarp();
  if (lane == 0) wcnt[w] = base + __popc(bal);
  __syncwarp();
}

__device__ __forceinline__ void vol_offsets(const int* wcnt, int* woff) {
  if (threadIdx.x == 0) {
    woff[0] = 0;
    for (int w = 0; w < kVolWarps; w++) woff[w + 1] = woff[w] + wcnt[w];
  }
}

__device__ __forceinline__ int vol_entry(const int* ent, const int* woff, int e) {
  int w = 0;
  while (woff[w + 1] <= e) w++;
  return ent[w * kVolSeg + (e - woff[w])];
}

// FP64 pair term with the blending square roots taken per atom
// (sqrt|s_a| sqrt|s_b| for sqrt|s_a s_b|, equal to within an ulp) and one
// reciprocal square root per pair (1/r and 1/r^2 = (1/r)^2 within a few
// ulps of the division and square root of the reference's arithmetic, at
// about half their FP64 cost); zero at r2 == 0 as the reference.
__device__ __forceinline__ double pair64f(double r2, double rsa, double rsb, double rea,
                                          double reb, double qq) {
  if (r2 == 0.0) return 0.0;
  const double ir = rsqrt(r2);
  const double ir2 = ir * ir;
  const double sg = rsa * rsb;
  const double s2 = sg * sg * ir2;
  const double s6 = s2 * s2 * s2;
  return 4.0 * (rea * reb) * (s6 * s6 - s6) + qq * ir;
}

// Chains a pair-sum pass evaluates: pass 0 the due non-mixed chains, pass 1
// the mixed chains whose double-float re-take was still too close to call
// (state 5), pass 2 the chains whose energy at their current box is wanted
// (one volume only).
__device__ __forceinline__ bool vol_take64(const VolMove& v, const ChainHdr& H, int pass) {
  if (pass == 2) return v.state == 1;  // a chain's energy at its current box
  return pass == 0 ? (v.state == 1 && !H.vol_mixed) : v.state == 5;
}

// The chains of a volume phase in state `want`, compacted: list[0] = their
// count k, list[1] = their molecules, then at list + 2, + 2 + cap and
// + 2 + 2 cap (cap = the phase's chain count) each one's slot, first pool
// molecule and molecule prefix sum (pref[k] = the total).  One warp.
__global__ void k_vol_list(Pool P, const VolMove* vm, MolRanges R, int nc, int want, int* list) {
  const int lane = threadIdx.x;
  if (lane >= 32) return;
  int k = 0, total = 0;
  const unsigned lt = (1u << lane) - 1u;
  for (int c0 = 0; c0 < nc; c0 += 32) {
    const int i = c0 + lane;
    int slot = 0, n = 0;
    bool flag = false;
    if (i < nc) {
      slot = range_chain(R, i);
      flag = vm[slot].state == want;
      if (flag) n = P.hdr[slot].n_mol;
    }
    int incl = n;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const int v = __shfl_up_sync(~0u, incl, off);
      if (lane >= off) incl += v;
    }
    const unsigned bal = __ballot_sync(~0u, flag);
    if (flag) {
      const int pos = k + __popc(bal & lt);
      list[2 + pos] = slot;
      list[2 + nc + pos] = P.hdr[slot].mol0;
      list[2 + 2 * nc + pos] = total + incl - n;
    }
    total += __shfl_sync(~0u, incl, 31);
    k += __popc(bal);
  }
  if (lane == 0) {
    list[0] = k;
    list[1] = total;
    list[2 + 2 * nc + k] = total;
  }
}

// E(m, j > m) of pool molecule m at V (.x) and V' (.y) with FP64 pair terms
// (the reference's, SimulationStep.cpp:344-375, with the blending roots per
// atom).  Candidates from the cell stencil, screened and compacted in
// chunks (vol_screen: the FP64 test's in-range set exactly).
__device__ __forceinline__ void vol_f64_mol(const Pool& P, const int* mol_chain,
                                            const VolMove* vm, int m, double2* emol2,
                                            int pass) {
  __shared__ double sx[3][kMaxA];
  __shared__ double sq[3][kMaxA];
  __shared__ int spa[kMaxP];
  __shared__ double2 red[kVolThreads];
  __shared__ VcStencil S;
  __shared__ VolBox vb[2];
  __shared__ float4 so[kMaxA];
  __shared__ int ent[kVolChunk];
  __shared__ int wcnt[kVolWarps], woff[kVolWarps + 1];
  const int c = mol_chain[m];
  const VolMove& v = vm[c];
  const ChainHdr& H = P.hdr[c];
  if (!vol_take64(v, H, pass)) return;
  const int nvol = pass == 2 ? 1 : 2;
  vc_stencil(P, H, m, S);
  if (threadIdx.x < 2) vb[threadIdx.x] = v.box[threadIdx.x];
  const int a0 = P.mstart[m], len = P.mlen[m] & 255;
  const int2 pi = P.mpi[m];
  const uint4 Am = P.mfix[m];
  for (int i = threadIdx.x; i < len; i += blockDim.x) {
    const float4 o = P.aoff[a0 + i];
    so[i] = o;
    // positions relative to the molecule's anchor (rigid: both volumes)
    sx[0][i] = (double)o.x;
    sx[1][i] = (double)o.y;
    sx[2][i] = (double)o.z;
    const double sg = P.sig[a0 + i], ep = P.eps[a0 + i];
    // dummy sites (sigma or epsilon < 0) are skipped: marked by -1
    sq[0][i] = (sg >= 0 && ep >= 0) ? sqrt(sg) : -1.0;
    sq[1][i] = (sg >= 0 && ep >= 0) ? sqrt(ep) : -1.0;
    sq[2][i] = P.q[a0 + i] * kCoulomb;
  }
  for (int k = threadIdx.x; k < pi.y; k += blockDim.x) spa[k] = P.pidx[pi.x + k] - a0;
  __syncthreads();
  const float reach2 = v.reach * v.reach;
  const float sf = v.sf;
  const float rad_m = P.mrad[m];
  const int maxlen = H.max_len;
  double eo = 0.0, en = 0.0;
  const int n_cand = S.pref[S.n];
  int kc = 0;
  for (int c0 = 0; c0 < n_cand; c0 += kVolChunk) {
    // screen: in-range flags of this chunk's candidates, compacted per warp
    for (int r = 0; r < kVolChunk / kVolThreads; r++) {
      const int t = c0 + r * kVolThreads + (int)threadIdx.x;
      int f = 0, j = 0;
      if (t < n_cand) {
        j = vc_candidate(P, S, t, kc);
        if (vc_takes(S, kc, j, m)) f = vol_screen(P, H, vb, so, spa, pi.y, Am, j, reach2, sf, 0, nvol);
      }
      vol_append(ent, wcnt, j, f, r);
    }
    __syncthreads();
    vol_offsets(wcnt, woff);
    __syncthreads();
    // pairs: one (neighbour, neighbour atom) item per thread
    const int items = woff[kVolWarps] * maxlen;
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
      const int e = it / maxlen, bi = it - e * maxlen;
      const int jf = vol_entry(ent, woff, e);
      const int j = jf & kVolJMask, f = jf >> kVolFShift;
      const int b0 = P.mstart[j], lenj = P.mlen[j] & 255;
      if (bi >= lenj) continue;
      const int bb = b0 + bi;
      const double sb = P.sig[bb], eb = P.eps[bb], qb = P.q[bb];
      if (!(sb >= 0 && eb >= 0)) continue;
      const double rsb = sqrt(sb), reb = sqrt(eb);
      const float4 ob = P.aoff[bb];
      const uint4 Aj = P.mfix[j];
      const float rr = rad_m + P.mrad[j];
#pragma unroll
      for (int w = 0; w < 2; w++) {
        if (!(f & (1 << w))) continue;
        const VolBox& B = vb[w];
        // b relative to m's anchor: the anchors' minimum-image difference
        // (fixed point) at this volume plus b's offset
        const int d[3] = {(int)(Aj.x - Am.x), (int)(Aj.y - Am.y), (int)(Aj.z - Am.z)};
        const double bx = (double)d[0] * (B.L[0] * 0x1p-32) + (double)ob.x;
        const double by = (double)d[1] * (B.L[1] * 0x1p-32) + (double)ob.y;
        const double bz = (double)d[2] * (B.L[2] * 0x1p-32) + (double)ob.z;
        // every pair within half an edge: no image to take
        const bool wrap = fabsf((float)d[0] * B.fxs[0]) + rr > 0.5f * B.Lf[0] - 1e-3f ||
                          fabsf((float)d[1] * B.fxs[1]) + rr > 0.5f * B.Lf[1] - 1e-3f ||
                          fabsf((float)d[2] * B.fxs[2]) + rr > 0.5f * B.Lf[2] - 1e-3f;
        double acc = 0.0;
        for (int i = 0; i < len; i++) {
          const double rsa = sq[0][i];
          if (rsa < 0) continue;
          double dx = bx - sx[0][i], dy = by - sx[1][i], dz = bz - sx[2][i];
          if (wrap) {
            dx = make_periodic(dx, B.L[0]);
            dy = make_periodic(dy, B.L[1]);
            dz = make_periodic(dz, B.L[2]);
          }
          const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)),
                                      __dmul_rn(dz, dz));
          acc += pair64f(r2, rsa, rsb, sq[1][i], reb, sq[2][i] * qb);
        }
        if (w == 0) eo += acc; else en += acc;
      }
    }
    __syncthreads();
  }
  red[threadIdx.x] = make_double2(eo, en);
  __syncthreads();
  for (int off = blockDim.x >> 1; off > 0; off >>= 1) {
    if ((int)threadIdx.x < off) {
      red[threadIdx.x].x += red[threadIdx.x + off].x;
      red[threadIdx.x].y += red[threadIdx.x + off].y;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) emol2[m] = red[0];
}


__global__ void __launch_bounds__(kVolThreads, 4) k_vol_pair_sums(Pool P, const int* mol_chain,
                                                               const VolMove* vm, int m_begin,
                                                               MolRanges R, double2* emol2,
                                                               int pass) {
  vol_f64_mol(P, mol_chain, vm, range_mol(R, m_begin, blockIdx.x), emol2, pass);
}

// The molecules of the chains a volume list holds (k_vol_list), grid-strided.
__device__ __forceinline__ int list_mol(const int* list, int cap, int b) {
  const int cnt = list[0];
  const int* m0 = list + 2 + cap;
  const int* pref = list + 2 + 2 * cap;
  int lo = 0, hi = cnt - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (pref[mid] <= b) lo = mid; else hi = mid - 1;
  }
  return m0[lo] + (b - pref[lo]);
}

// FP64 re-take (pass 1: chains in state 5) over the listed chains only.
__global__ void __launch_bounds__(kVolThreads, 4) k_vol_pair_sums_list(Pool P,
                                                                    const int* mol_chain,
                                                                    const VolMove* vm,
                                                                    const int* list, int cap,
                                                                    double2* emol2) {
  const int total = list[1];
  for (int b = blockIdx.x; b < total; b += gridDim.x) {
    vol_f64_mol(P, mol_chain, vm, list_mol(list, cap, b), emol2, 1);
    __syncthreads();
  }
}

// E(m, j > m) at V (.x) and V' (.y) of a chain whose FP32 volume decision
// was too close to call (state 4), with pair terms in double-float
// arithmetic from the FP64 rows' parameters and the exact anchor-relative
// positions (anchor difference as a double-float plus FP32 offsets); eabs2
// gets the sums of the terms' magnitudes for the re-take's own bound.  The
// in-range set is the FP64 test's (vol_screen), the arithmetic the
// reference's (SimulationStep.cpp:344-375, BruteForceStep.cpp:61-76) to
// about 1e-13 relative, at a fraction of the FP64 pipe's cost.
__device__ __forceinline__ void vol_df_mol(const Pool& P, const int* mol_chain,
                                           const VolMove* vm, int m, double2* emol2,
                                           double2* eabs2) {
  __shared__ float4 so[kMaxA];
  __shared__ df ssg[kMaxA], sep4[kMaxA], sqc[kMaxA];
  __shared__ int spa[kMaxP];
  __shared__ VolBox vb[2];
  __shared__ float wred[kVolWarps][6];
  __shared__ VcStencil S;
  __shared__ int ent[kVolChunk];
  __shared__ int wcnt[kVolWarps], woff[kVolWarps + 1];
  const int c = mol_chain[m];
  const VolMove& v = vm[c];
  const ChainHdr& H = P.hdr[c];
  if (v.state != 4 && v.state != 6) return;
  // state 6 re-takes U(V') only (.x stays 0)
  const int w0 = v.state == 6 ? 1 : 0, nvol = v.state == 6 ? 1 : 2;
  vc_stencil(P, H, m, S);
  const int a0 = P.mstart[m], len = P.mlen[m] & 255;
  const int2 pi = P.mpi[m];
  const uint4 Am = P.mfix[m];
  for (int i = threadIdx.x; i < len; i += blockDim.x) {
    so[i] = P.aoff[a0 + i];
    const double sg = P.sig[a0 + i], ep = P.eps[a0 + i];
    // dummy sites (sigma or epsilon < 0) are skipped: sigma marked -1
    const bool real = sg >= 0 && ep >= 0;
    ssg[i] = real ? df_of(sg) : df{-1.0f, 0.0f};
    sep4[i] = df_of(real ? 4.0 * sqrt(ep) : 0.0);
    sqc[i] = df_of(P.q[a0 + i] * kCoulomb);
  }
  for (int k = threadIdx.x; k < pi.y; k += blockDim.x) spa[k] = P.pidx[pi.x + k] - a0;
  if (threadIdx.x < 2) vb[threadIdx.x] = v.box[threadIdx.x];
  __syncthreads();
  const float reach2 = v.reach * v.reach;
  const float sf = v.sf;
  const float rad_m = P.mrad[m];
  df acc[2] = {{0.f, 0.f}, {0.f, 0.f}};
  float ab[2] = {0.f, 0.f};
  const int maxlen = H.max_len;
  const int n_cand = S.pref[S.n];
  int kc = 0;
  for (int c0 = 0; c0 < n_cand; c0 += kVolChunk) {
    for (int r = 0; r < kVolChunk / kVolThreads; r++) {
      const int t = c0 + r * kVolThreads + (int)threadIdx.x;
      int f = 0, j = 0;
      if (t < n_cand) {
        j = vc_candidate(P, S, t, kc);
        if (vc_takes(S, kc, j, m))
          f = vol_screen(P, H, vb, so, spa, pi.y, Am, j, reach2, sf, w0, nvol);
      }
      vol_append(ent, wcnt, j, f, r);
    }
    __syncthreads();
    vol_offsets(wcnt, woff);
    __syncthreads();
    const int items = woff[kVolWarps] * maxlen;
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
      const int e = it / maxlen, bi = it - e * maxlen;
      const int jf = vol_entry(ent, woff, e);
      const int j = jf & kVolJMask, f = jf >> kVolFShift;
      const int lenj = P.mlen[j] & 255;
      if (bi >= lenj) continue;
      const int bb = P.mstart[j] + bi;
      const double sgb = P.sig[bb], epb = P.eps[bb];
      if (!(sgb >= 0 && epb >= 0)) continue;
      const df sb = df_of(sgb), eb = df_of(epb), qb = df_of(P.q[bb]);
      // sqrt(eps_b) = eps_b / sqrt(eps_b)
      const df reb = eb.h > 0.f ? df_mul(eb, df_rsqrt(eb)) : df{0.f, 0.f};
      const float4 ob = P.aoff[bb];
      const uint4 Aj = P.mfix[j];
      const float rr = rad_m + P.mrad[j];
#pragma unroll
      for (int w = 0; w < 2; w++) {
        if (!(f & (1 << w))) continue;
        const VolBox& B = vb[w];
        float3 Dh, Dl;
        vol_fixdiff(Aj, Am, B, Dh, Dl);
        // b relative to m's anchor, double-float
        const df bx = df_add(df_two_sum(Dh.x, ob.x), {Dl.x, 0.f});
        const df by = df_add(df_two_sum(Dh.y, ob.y), {Dl.y, 0.f});
        const df bz = df_add(df_two_sum(Dh.z, ob.z), {Dl.z, 0.f});
        const bool wrap = fabsf(Dh.x) + rr > 0.5f * B.Lf[0] - 1e-3f ||
                          fabsf(Dh.y) + rr > 0.5f * B.Lf[1] - 1e-3f ||
                          fabsf(Dh.z) + rr > 0.5f * B.Lf[2] - 1e-3f;
        for (int i = 0; i < len; i++) {
          const df sa = ssg[i];
          if (sa.h < 0.f) continue;
          const float4 oa = so[i];
          df d[3] = {df_sub(bx, {oa.x, 0.f}), df_sub(by, {oa.y, 0.f}), df_sub(bz, {oa.z, 0.f})};
          if (wrap) {
#pragma unroll
            for (int k = 0; k < 3; k++) {
              // SimCalcs::makePeriodic on the double-float difference
              const double L = B.L[k];
              const double x = (double)d[k].h + (double)d[k].l;
              if (x < -0.5 * L) d[k] = df_add(d[k], df_of(L));
              else if (x > 0.5 * L) d[k] = df_sub(d[k], df_of(L));
            }
          }
          const df r2 = df_add(df_add(df_mul(d[0], d[0]), df_mul(d[1], d[1])), df_mul(d[2], d[2]));
          if (!(r2.h > 0.f)) continue;
          const df ir = df_rsqrt(r2);
          const df ir2 = df_mul(ir, ir);
          const df s2 = df_mul(df_mul(sa, sb), ir2);
          const df s6 = df_mul(df_mul(s2, s2), s2);
          const df lj = df_mul(df_mul(sep4[i], reb), df_sub(df_mul(s6, s6), s6));
          const df cl = df_mul(df_mul(sqc[i], qb), ir);
          acc[w] = df_add(acc[w], df_add(lj, cl));
          ab[w] += fabsf(lj.h) + fabsf(cl.h);
        }
      }
    }
    __syncthreads();
  }
  // reduction: warp butterflies in double-float, then the warps in order
  for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
    for (int w = 0; w < 2; w++) {
      const df o = {__shfl_xor_sync(~0u, acc[w].h, off), __shfl_xor_sync(~0u, acc[w].l, off)};
      acc[w] = df_add(acc[w], o);
      ab[w] += __shfl_xor_sync(~0u, ab[w], off);
    }
  }
  if ((threadIdx.x & 31) == 0) {
    const int wi = threadIdx.x >> 5;
    wred[wi][0] = acc[0].h; wred[wi][1] = acc[0].l; wred[wi][2] = acc[1].h;
    wred[wi][3] = acc[1].l; wred[wi][4] = ab[0]; wred[wi][5] = ab[1];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    df s0 = {0.f, 0.f}, s1 = {0.f, 0.f};
    float a0s = 0.f, a1s = 0.f;
    for (int wi = 0; wi < kVolWarps; wi++) {
      s0 = df_add(s0, {wred[wi][0], wred[wi][1]});
      s1 = df_add(s1, {wred[wi][2], wred[wi][3]});
      a0s += wred[wi][4];
      a1s += wred[wi][5];
    }
    emol2[m] = make_double2((double)s0.h + (double)s0.l, (double)s1.h + (double)s1.l);
    eabs2[m] = make_double2((double)a0s, (double)a1s);
  }
}


__global__ void __launch_bounds__(kVolThreads) k_vol_pair_sums_df(Pool P, const int* mol_chain,
                                                                  const VolMove* vm,
                                                                  const int* list, int cap,
                                                                  double2* emol2, double2* eabs2) {
  const int total = list[1];
  for (int b = blockIdx.x; b < total; b += gridDim.x) {
    vol_df_mol(P, mol_chain, vm, list_mol(list, cap, b), emol2, eabs2);
    __syncthreads();
  }
}

// FP32 pair terms of neighbour atom b (at bx + lx etc. relative to the moved
// molecule's anchor, double-float) with every atom of the molecule staged in
// so/sq.  WRAP takes each pair's own minimum image; without it the pair
// distances are used as they are, which gives the same r2 bit for bit when
// every |d| stays below half an edge (the caller's |D| + radii test).
template <bool WRAP>
__device__ __forceinline__ void vol_atoms32(const float4* so, const float2* sq, int len, float bx,
                                            float by, float bz, float lx, float ly, float lz,
                                            float sig_b, float2 qb, const VolBox& B, float& e32,
                                            float& a32) {
  for (int i = 0; i < len; i++) {
    const float4 a4 = so[i];
    const float2 ea = sq[i];
    float dx = (bx - a4.x) + lx, dy = (by - a4.y) + ly, dz = (bz - a4.z) + lz;
    if (WRAP) {
      dx = wrapf(dx, B.Lf[0]);
      dy = wrapf(dy, B.Lf[1]);
      dz = wrapf(dz, B.Lf[2]);
    }
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    if (!(r2 > 0.f)) continue;
    const float lj = lj32(rcp_nr(r2), a4.w, sig_b, ea.x, qb.x);
    const float cl = (ea.y * qb.y) * rsqrt_nr(r2);
    e32 += lj + cl;
    a32 += fabsf(lj) + fabsf(cl);
  }
}

// E(V') - E(V) of neighbour atom b with every atom of molecule m, for a pair
// of molecules in range at both volumes that uses the anchors' image at
// both.  (bx..lz) is b relative to m's anchor at V (double-float), (ex, ey,
// ez) the change of the anchor difference from V to V', (s' - s) D: every
// atom pair's displacement changes by it, so r'^2 - r^2 = 2 d.delta +
// delta^2, a small number with a small relative error, and
//   1/r' - 1/r      = -(r'^2 - r^2) / (r r' (r + r')),
//   t' - t          = -sigma^2 (r'^2 - r^2) / (r^2 r'^2),   t = sigma^2/r^2,
//   t'^3 - t^3      = (t' - t)(t'^2 + t' t + t^2),  t'^6 - t^6 = (t'^3 - t^3)(t'^3 + t^3)
// give each pair's change without the cancellation of two FP32 energies.
// a32 gets the magnitude that bounds its rounding: the same expressions with
// |r'^2 - r^2| replaced by the sum of its terms' magnitudes.  A pair that
// coincides at either volume is taken as the difference of the two direct
// terms (the reference skips r = 0).
__device__ __forceinline__ void vol_atoms_delta(const float4* so, const float2* sq, int len,
                                                float bx, float by, float bz, float lx, float ly,
                                                float lz, float ex, float ey, float ez,
                                                float sig_b, float2 qb, float& e32, float& a32) {
  for (int i = 0; i < len; i++) {
    const float4 a4 = so[i];
    const float2 ea = sq[i];
    const float dx = (bx - a4.x) + lx, dy = (by - a4.y) + ly, dz = (bz - a4.z) + lz;
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    const float q = fmaf(fmaf(2.f, dx, ex), ex, fmaf(fmaf(2.f, dy, ey), ey, fmaf(2.f, dz, ez) * ez));
    const float r2p = r2 + q;
    const float ee = ea.x * qb.x, cq = ea.y * qb.y, s2 = a4.w * sig_b;
    if (!(r2 > 0.f) || !(r2p > 0.f)) {
      // degenerate pair: the two direct terms (each only where r > 0)
      if (r2p > 0.f) {
        const float lj = lj32(rcp_nr(r2p), a4.w, sig_b, ea.x, qb.x), cl = cq * rsqrt_nr(r2p);
        e32 += lj + cl;
        a32 += fabsf(lj) + fabsf(cl);
      }
      if (r2 > 0.f) {
        const float lj = lj32(rcp_nr(r2), a4.w, sig_b, ea.x, qb.x), cl = cq * rsqrt_nr(r2);
        e32 -= lj + cl;
        a32 += fabsf(lj) + fabsf(cl);
      }
      continue;
    }
    const float qa = fabsf(2.f * dx * ex) + fabsf(2.f * dy * ey) + fabsf(2.f * dz * ez) +
                     fmaf(ex, ex, fmaf(ey, ey, ez * ez));
    const float ir = rsqrt_nr(r2), irp = rsqrt_nr(r2p);
    const float ir2 = rcp_nr(r2), ir2p = rcp_nr(r2p);
    const float w = ir * irp * rcp_approx(fmaf(r2, ir, r2p * irp));  // 1 / (r r' (r + r'))
    const float dcl = cq * (-q * w);
    const float t = s2 * ir2;
    const float g = s2 * ir2 * ir2p;                                  // sigma^2 / (r^2 r'^2)
    const float tp = fmaf(-q, g, t);
    const float t3 = t * t * t, tp3 = tp * tp * tp;
    const float d3 = (-q * g) * fmaf(tp, tp, fmaf(tp, t, t * t));
    const float dlj = ee * (d3 * (tp3 + t3) - d3);
    e32 += dlj + dcl;
    const float tm = fmaxf(t, tp), tm2 = tm * tm;
    a32 += qa * (fabsf(cq) * w + fabsf(ee) * g * tm2 * (6.f * tm2 * tm + 3.f));
  }
}

// E(m, j > m) of a mixed chain's molecule m: with init, at V (.x; any chain
// in state 1); for a volume move, the change E(V') - E(V) (.y), the pairs in
// range at both volumes by vol_atoms_delta, the others (crossing the cutoff,
// or taking their own images) as the difference of the direct terms.  FP32
// pair terms (the chain kernel's arithmetic) summed in double-float; eabs2
// gets the sums of the magnitudes that bound their rounding.  The in-range
// test is the FP32 screen with the FP64 re-test inside its guard band: the
// FP64 test's set exactly.
__global__ void __launch_bounds__(kVolThreads, 8) k_vol_pair_sums32(Pool P, const int* mol_chain,
                                                                 const VolMove* vm, int m_begin,
                                                                 MolRanges R, double2* emol2,
                                                                 double2* eabs2, int init) {
  __shared__ float4 so[kMaxA];
  __shared__ float2 sq[kMaxA];
  __shared__ int spa[kMaxP];
  __shared__ VolBox vb[2];
  __shared__ float wred[kVolWarps][6];
  __shared__ VcStencil S;
  __shared__ int ent[kVolChunk];
  __shared__ int wcnt[kVolWarps], woff[kVolWarps + 1];
  const int m = range_mol(R, m_begin, blockIdx.x);
  const int c = mol_chain[m];
  const VolMove& v = vm[c];
  const ChainHdr& H = P.hdr[c];
  // init: a chain's energy at its current box; else dU of a mixed move
  if (!(v.state == 1 && (H.vol_mixed || init))) return;
  const bool delta = !init;
  __shared__ float sm1[3];   // s - 1 per edge, s = L'/L
  if (delta && threadIdx.x < 3)
    sm1[threadIdx.x] = (float)(v.box[1].L[threadIdx.x] / v.box[0].L[threadIdx.x] - 1.0);
  vc_stencil(P, H, m, S);
  const int a0 = P.mstart[m], len = P.mlen[m] & 255;
  const int2 pi = P.mpi[m];
  const uint4 Am = P.mfix[m];
  for (int i = threadIdx.x; i < len; i += blockDim.x) {
    so[i] = P.aoff[a0 + i];
    sq[i] = P.aeq[a0 + i];
  }
  for (int k = threadIdx.x; k < pi.y; k += blockDim.x) spa[k] = P.pidx[pi.x + k] - a0;
  if (threadIdx.x < 2) vb[threadIdx.x] = v.box[threadIdx.x];
  __syncthreads();
  const float reach2 = v.reach * v.reach;
  const float sf = v.sf;
  const float rad_m = P.mrad[m];
  float eh[2] = {0.f, 0.f}, el[2] = {0.f, 0.f}, ab[2] = {0.f, 0.f};
  const int maxlen = H.max_len;
  const int n_cand = S.pref[S.n];
  int kc = 0;
  for (int c0 = 0; c0 < n_cand; c0 += kVolChunk) {
    for (int r = 0; r < kVolChunk / kVolThreads; r++) {
      const int t = c0 + r * kVolThreads + (int)threadIdx.x;
      int f = 0, j = 0;
      if (t < n_cand) {
        j = vc_candidate(P, S, t, kc);
        if (vc_takes(S, kc, j, m))
          f = vol_screen(P, H, vb, so, spa, pi.y, Am, j, reach2, sf, 0, delta ? 2 : 1);
      }
      vol_append(ent, wcnt, j, f, r);
    }
    __syncthreads();
    vol_offsets(wcnt, woff);
    __syncthreads();
    const int items = woff[kVolWarps] * maxlen;
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
      const int e = it / maxlen, bi = it - e * maxlen;
      const int jf = vol_entry(ent, woff, e);
      const int j = jf & kVolJMask, f = jf >> kVolFShift;
      const int lenj = P.mlen[j] & 255;
      if (bi >= lenj) continue;
      const int bb = P.mstart[j] + bi;
      const float4 ob = P.aoff[bb];
      const float2 qb = P.aeq[bb];
      const uint4 Aj = P.mfix[j];
      const float rad_j = P.mrad[j];
      const float rr = rad_m + rad_j;
      if (delta && f == 3) {
        float3 Dh, Dl, Dh1, Dl1;
        vol_fixdiff(Aj, Am, vb[0], Dh, Dl);
        vol_fixdiff(Aj, Am, vb[1], Dh1, Dl1);
        const bool wrap = fabsf(Dh.x) + rr > 0.5f * vb[0].Lf[0] - 1e-3f ||
                          fabsf(Dh.y) + rr > 0.5f * vb[0].Lf[1] - 1e-3f ||
                          fabsf(Dh.z) + rr > 0.5f * vb[0].Lf[2] - 1e-3f ||
                          fabsf(Dh1.x) + rr > 0.5f * vb[1].Lf[0] - 1e-3f ||
                          fabsf(Dh1.y) + rr > 0.5f * vb[1].Lf[1] - 1e-3f ||
                          fabsf(Dh1.z) + rr > 0.5f * vb[1].Lf[2] - 1e-3f;
        if (!wrap) {
          const float bx = Dh.x + ob.x, by = Dh.y + ob.y, bz = Dh.z + ob.z;
          const float lx = ((Dh.x - (bx - (bx - Dh.x))) + (ob.x - (bx - Dh.x))) + Dl.x;
          const float ly = ((Dh.y - (by - (by - Dh.y))) + (ob.y - (by - Dh.y))) + Dl.y;
          const float lz = ((Dh.z - (bz - (bz - Dh.z))) + (ob.z - (bz - Dh.z))) + Dl.z;
          float e32 = 0.f, a32 = 0.f;
          vol_atoms_delta(so, sq, len, bx, by, bz, lx, ly, lz, Dh.x * sm1[0], Dh.y * sm1[1],
                          Dh.z * sm1[2], ob.w, qb, e32, a32);
          ff_add(eh[1], el[1], e32);
          ab[1] += a32;
          continue;
        }
      }
#pragma unroll
      for (int w = 0; w < 2; w++) {
        if (!(f & (1 << w))) continue;
        const VolBox& B = vb[w];
        float3 Dh, Dl;
        vol_fixdiff(Aj, Am, B, Dh, Dl);
        // b relative to m's anchor as a double-float: two-sum of D + o_b
        const float bx = Dh.x + ob.x, by = Dh.y + ob.y, bz = Dh.z + ob.z;
        const float lx = ((Dh.x - (bx - (bx - Dh.x))) + (ob.x - (bx - Dh.x))) + Dl.x;
        const float ly = ((Dh.y - (by - (by - Dh.y))) + (ob.y - (by - Dh.y))) + Dl.y;
        const float lz = ((Dh.z - (bz - (bz - Dh.z))) + (ob.z - (bz - Dh.z))) + Dl.z;
        float e32 = 0.f, a32 = 0.f;
        if (fabsf(Dh.x) + rr > 0.5f * B.Lf[0] - 1e-3f || fabsf(Dh.y) + rr > 0.5f * B.Lf[1] - 1e-3f ||
            fabsf(Dh.z) + rr > 0.5f * B.Lf[2] - 1e-3f)
          vol_atoms32<true>(so, sq, len, bx, by, bz, lx, ly, lz, ob.w, qb, B, e32, a32);
        else
          vol_atoms32<false>(so, sq, len, bx, by, bz, lx, ly, lz, ob.w, qb, B, e32, a32);
        // the change of a volume move: +E(V') - E(V), both into .y
        const int wo = delta ? 1 : w;
        ff_add(eh[wo], el[wo], (delta && w == 0) ? -e32 : e32);
        ab[wo] += a32;
      }
    }
    __syncthreads();
  }
  // double-float reduction (warp butterflies, then the warps in order); one
  // conversion to FP64 per molecule
  for (int off = 16; off > 0; off >>= 1) {
    for (int w = 0; w < 2; w++) {
      const float h = __shfl_xor_sync(~0u, eh[w], off), l = __shfl_xor_sync(~0u, el[w], off);
      ff_add2(eh[w], el[w], h, l);
      ab[w] += __shfl_xor_sync(~0u, ab[w], off);
    }
  }
  if ((threadIdx.x & 31) == 0) {
    const int wi = threadIdx.x >> 5;
    wred[wi][0] = eh[0]; wred[wi][1] = el[0]; wred[wi][2] = eh[1];
    wred[wi][3] = el[1]; wred[wi][4] = ab[0]; wred[wi][5] = ab[1];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float h0 = 0.f, l0 = 0.f, h1 = 0.f, l1 = 0.f, a0 = 0.f, a1 = 0.f;
    for (int wi = 0; wi < kVolWarps; wi++) {
      ff_add2(h0, l0, wred[wi][0], wred[wi][1]);
      ff_add2(h1, l1, wred[wi][2], wred[wi][3]);
      a0 += wred[wi][4];
      a1 += wred[wi][5];
    }
    emol2[m] = make_double2((double)h0 + (double)l0, (double)h1 + (double)l1);
    eabs2[m] = make_double2((double)a0, (double)a1);
  }
}

// Ordered per-chain sums of emol2 (and, for FP32 energies, of the term
// magnitudes eabs2) for the chains in state `want`.
constexpr int kVolSumThreads = 1024;

__global__ void __launch_bounds__(kVolSumThreads) k_vol_sums(Pool P, const VolMove* vm,
                                                             const double2* emol2,
                                                             const double2* eabs2, double2* out,
                                                             double2* out_abs, MolRanges R,
                                                             int want) {
  __shared__ double2 red[kVolSumThreads];
  __shared__ double2 rab[kVolSumThreads];
  const int c = range_chain(R, blockIdx.x);
  if (vm[c].state != want) return;
  const ChainHdr& H = P.hdr[c];
  const bool mixed = want == 1 || want == 4 || want == 6;
  double2 acc = make_double2(0.0, 0.0), ab = make_double2(0.0, 0.0);
  for (int i = threadIdx.x; i < H.n_mol; i += blockDim.x) {
    acc.x += emol2[H.mol0 + i].x;
    acc.y += emol2[H.mol0 + i].y;
    if (mixed) {
      ab.x += eabs2[H.mol0 + i].x;
      ab.y += eabs2[H.mol0 + i].y;
    }
  }
  red[threadIdx.x] = acc;
  rab[threadIdx.x] = ab;
  __syncthreads();
  for (int off = blockDim.x >> 1; off > 0; off >>= 1) {
    if ((int)threadIdx.x < off) {
      red[threadIdx.x].x += red[threadIdx.x + off].x;
      red[threadIdx.x].y += red[threadIdx.x + off].y;
      rab[threadIdx.x].x += rab[threadIdx.x + off].x;
      rab[threadIdx.x].y += rab[threadIdx.x + off].y;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[c] = red[0];
    out_abs[c] = mixed ? rab[0] : make_double2(0.0, 0.0);
  }
}

// The isobaric criterion; an accepted move installs the new box.
// Pass 0 decides the due chains (a mixed chain whose FP32 argument lies
// within its error bound of ln u is marked state 6 instead); pass 3 decides
// state 6 on the double-float U(V') (still too close: state 4), pass 1 state
// 4 on double-float totals at both volumes (still too close: state 5), pass
// 2 state 5 on FP64 totals.
__global__ void k_vol_decide(Pool P, VolMove* vm, const double2* esum, const double2* eabs,
                             mcgpu_vol_trace* trace, int trace_slot, int trace_stride,
                             MolRanges R, int n_items, int pass) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_items) return;
  const int c = range_chain(R, i);
  VolMove v = vm[c];
  const int want = pass == 1 ? 4 : (pass == 2 ? 5 : 6);
  if (pass == 0 ? (v.state != 1 && v.state != 2) : v.state != want) return;
  ChainHdr& H = P.hdr[c];
  double e_old = H.energy, e_new = 0.0;
  int ok = 0;
  if (v.state != 2) {
    // a mixed move's dU is summed pair by pair in FP32 (esum.y; its bound
    // does not involve the running energy U(V)); too close to call, U(V') is
    // taken in double-float with U(V) the running energy (state 6), then both
    // totals in double-float (state 4), then both in FP64 (state 5); an FP64
    // chain has both FP64 totals
    const bool mixed = v.state == 1 && H.vol_mixed;
    const bool vprime = v.state == 6;
    const bool dfl = v.state == 4;
    e_old = (mixed || vprime) ? H.energy : esum[c].x;
    e_new = mixed ? H.energy + esum[c].y : esum[c].y;
    const double vo = H.L[0] * H.L[1] * H.L[2];
    const double vn = v.L[0] * v.L[1] * v.L[2];
    // the tail correction E_LRC = lrc_v / V changes with the volume
    const double d_lrc = H.lrc_v / vn - H.lrc_v / vo;
    const double du = mixed ? esum[c].y : e_new - e_old;
    const double arg = -(du + d_lrc + H.pressure * (vn - vo)) / H.kT +
                       (double)(H.n_mol + 1) * v.dlnv;
    double err_old = 0.0, err_new = 0.0;
    if (mixed) {
      err_new = kTieRel * eabs[c].y;   // the bound of dU
    } else if (vprime) {
      err_old = H.run_err;
      err_new = kDfRel * eabs[c].y;
    } else if (dfl) {
      err_old = kDfRel * eabs[c].x;
      err_new = kDfRel * eabs[c].y;
    }
    if (mixed || vprime || dfl) {
      // |error of dU| <= err_old + err_new
      const double bound = (err_old + err_new + 1e-12 * (fabs(e_old) + fabs(e_new))) / H.kT;
      if (fabs(arg - log(v.u)) <= bound + 1e-12) {
        v.state = mixed ? 6 : (vprime ? 4 : 5);
        v.fp64 = mixed ? 2 : 1;   // 2: only U(V') is taken again
        vm[c] = v;
        return;
      }
    }
    ok = (arg >= 0.0) || (exp(arg) >= v.u);
    if (ok) {
      H.energy = e_new;
      // a mixed move adds dU to the running energy and its bound to run_err;
      // the other tiers install a fresh total with its own bound
      H.run_err = mixed ? H.run_err + err_new : err_new;
    } else if (!mixed && !vprime) {
      H.energy = e_old;
      H.run_err = err_old;
    }
  }
  H.vol_tried++;
  H.vol_step = (long long)H.step;
  if (v.fp64) H.vol_fp64++;
  if (ok) {
    hdr_set_box(H, v.L);
    H.vol_accepted++;
    H.nl_valid = 0;  // every centre moved: the Verlet list is rebuilt
    v.state = 3;
    vm[c] = v;
  }
  if (trace) {
    mcgpu_vol_trace t;
    t.step = (int64_t)H.step;
    t.accepted = ok;
    t.evaluated = v.state != 2;
    t.e_old = e_old;
    t.e_new = e_new;
    t.dlnv = v.dlnv;
    t.u = v.u;
    t.edge = H.L[0];
    t.fp64 = v.fp64;
    t.pad0 = 0;
    trace[(size_t)c * trace_stride + trace_slot] = t;
  }
}

// Screen positions of the primaries of every molecule of an accepting chain.
__global__ void k_vol_refresh(Pool P, const int* mol_chain, const VolMove* vm, int n_items,
                              MolRanges R) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n_items) return;
  const int m = range_mol(R, 0, b);
  const int c = mol_chain[m];
  if (vm[c].state != 3) return;
  const ChainHdr& H = P.hdr[c];
  const int2 pi = P.mpi[m];
  const uint4 A = P.mfix[m];
  for (int k = 0; k < pi.y; k++) {
    const double3 x = chain_pos3(A, P.aoff[P.pidx[pi.x + k]], H);
    P.ppos[pi.x + k] = wrap_pos(x.x, x.y, x.z, H);
  }
}

// A "volume move" to the chain's own box: state 1, both boxes the current
// one, so the cell grid and the pair kernels give the chain's energy.
__global__ void k_vol_self(Pool P, VolMove* vm, MolRanges R, int n_items) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_items) return;
  const int c = range_chain(R, i);
  const ChainHdr& H = P.hdr[c];
  VolMove v;
  for (int k = 0; k < 3; k++) v.L[k] = H.L[k];
  volbox_set(v.box[0], H.L, H.cutoff);
  v.box[1] = v.box[0];
  v.reach = vol_reach(H);
  v.sf = 1.0f;
  v.dlnv = 0.0;
  v.u = 0.0;
  v.fp64 = 0;
  v.state = H.n_mol > 0 ? 1 : 0;
  vm[c] = v;
}

__global__ void k_vol_self_energy(Pool P, const VolMove* vm, const double2* esum,
                                  const double2* esum_abs, MolRanges R, int n_items, int f64) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_items) return;
  const int c = range_chain(R, i);
  if (vm[c].state != 1) return;
  P.hdr[c].energy = esum[c].x;
  P.hdr[c].run_err = f64 ? 0.0 : kTieRel * esum_abs[c].x;
}

// Sets the running energy of the chains in act (all when act has no
// ranges) to their system energy, FP64 or FP32 pair terms (double-float
// sums), through the volume machinery; vm, emol2, eabs2, esum, esum_abs are
// scratch of the volume phase (the chains' own entries only).
cudaError_t launch_chain_energy(Pool P, const int* mol_chain, int n_mol_total, VolMove* vm,
                                double2* emol2, double2* eabs2, double2* esum, double2* esum_abs,
                                cudaStream_t st, MolRanges act, bool f64) {
  const int nc = act.act_slot ? act.n_act : P.n_chains;
  const int items = act.act_pref ? act.total : n_mol_total;
  if (nc == 0 || items == 0) return cudaSuccess;
  k_vol_self<<<(nc + 127) / 128, 128, 0, st>>>(P, vm, act, nc);
  const int gb = (items + 255) / 256;
  k_vc_grid<<<nc, 128, 0, st>>>(P, vm, act, nc);
  k_vc_count<<<gb, 256, 0, st>>>(P, mol_chain, vm, act, items);
  k_vc_scan<<<nc, 256, 0, st>>>(P, vm, act, nc);
  k_vc_scatter<<<gb, 256, 0, st>>>(P, mol_chain, vm, act, items);
  k_vc_sort<<<(items + kVcSortWarps - 1) / kVcSortWarps, 32 * kVcSortWarps, 0, st>>>(
        P, mol_chain, vm, act, items);
  const int chunk = act.act_pref ? items : (1 << 20);
  for (int m0 = 0; m0 < items; m0 += chunk) {
    const int n = items - m0 < chunk ? items - m0 : chunk;
    if (f64)
      k_vol_pair_sums<<<n, kVolThreads, 0, st>>>(P, mol_chain, vm, m0, act, emol2, 2);
    else
      k_vol_pair_sums32<<<n, kVolThreads, 0, st>>>(P, mol_chain, vm, m0, act, emol2, eabs2, 1);
  }
  k_vol_sums<<<nc, kVolSumThreads, 0, st>>>(P, vm, emol2, eabs2, esum, esum_abs, act, 1);
  k_vol_self_energy<<<(nc + 127) / 128, 128, 0, st>>>(P, vm, esum, esum_abs, act, nc, f64 ? 1 : 0);
  return cudaGetLastError();
}

// One volume phase on stream st (buffers sized for the pool).  has64 /
// has32: some due chain uses FP64 / FP32 pair energies (the other pair
// kernel is skipped).  With active ranges the work items are the ranges'
// molecules, numbered from 0; otherwise all pool molecules in chunks.
cudaError_t launch_volume_phase(Pool P, const int* mol_chain, int n_mol_total, VolMove* vm,
                                double2* emol2, double2* eabs2, double2* esum, double2* esum_abs,
                                int* vlist, mcgpu_vol_trace* trace, int trace_slot,
                                int trace_stride, cudaStream_t st, MolRanges act, bool has64,
                                bool has32) {
  const int nc = act.act_slot ? act.n_act : P.n_chains;
  if (nc == 0) return cudaSuccess;
  k_vol_propose<<<(nc + 127) / 128, 128, 0, st>>>(P, vm, act, nc);
  const int items = act.act_pref ? act.total : n_mol_total;
  if (items > 0) {
    const int gb = (items + 255) / 256;
    k_vc_grid<<<nc, 128, 0, st>>>(P, vm, act, nc);
    k_vc_count<<<gb, 256, 0, st>>>(P, mol_chain, vm, act, items);
    k_vc_scan<<<nc, 256, 0, st>>>(P, vm, act, nc);
    k_vc_scatter<<<gb, 256, 0, st>>>(P, mol_chain, vm, act, items);
    k_vc_sort<<<(items + kVcSortWarps - 1) / kVcSortWarps, 32 * kVcSortWarps, 0, st>>>(
        P, mol_chain, vm, act, items);
  }
  auto pairs = [&](bool f64, int pass) {
    if (items <= 0) return;
    if (act.act_pref) {
      if (f64)
        k_vol_pair_sums<<<items, kVolThreads, 0, st>>>(P, mol_chain, vm, 0, act, emol2, pass);
      else
        k_vol_pair_sums32<<<items, kVolThreads, 0, st>>>(P, mol_chain, vm, 0, act, emol2, eabs2, 0);
      return;
    }
    const int chunk = 1 << 20;
    for (int m0 = 0; m0 < items; m0 += chunk) {
      const int n = items - m0 < chunk ? items - m0 : chunk;
      if (f64)
        k_vol_pair_sums<<<n, kVolThreads, 0, st>>>(P, mol_chain, vm, m0, act, emol2, pass);
      else
        k_vol_pair_sums32<<<n, kVolThreads, 0, st>>>(P, mol_chain, vm, m0, act, emol2, eabs2, 0);
    }
  };
  if (has64) pairs(true, 0);
  if (has32) pairs(false, 0);
  k_vol_sums<<<nc, kVolSumThreads, 0, st>>>(P, vm, emol2, eabs2, esum, esum_abs, act, 1);
  k_vol_decide<<<(nc + 127) / 128, 128, 0, st>>>(P, vm, esum, esum_abs, trace, trace_slot,
                                                trace_stride, act, nc, 0);
  if (has32) {
    // too close to call in FP32: double-float re-take, and FP64 for what
    // is still too close after that
    // the re-takes run over the listed chains' molecules only (grid-strided)
    const int grid = kVolListGrid;
    k_vol_list<<<1, 32, 0, st>>>(P, vm, act, nc, 6, vlist);
    k_vol_pair_sums_df<<<grid, kVolThreads, 0, st>>>(P, mol_chain, vm, vlist, nc, emol2, eabs2);
    k_vol_sums<<<nc, kVolSumThreads, 0, st>>>(P, vm, emol2, eabs2, esum, esum_abs, act, 6);
    k_vol_decide<<<(nc + 127) / 128, 128, 0, st>>>(P, vm, esum, esum_abs, trace, trace_slot,
                                                  trace_stride, act, nc, 3);
    k_vol_list<<<1, 32, 0, st>>>(P, vm, act, nc, 4, vlist);
    k_vol_pair_sums_df<<<grid, kVolThreads, 0, st>>>(P, mol_chain, vm, vlist, nc, emol2, eabs2);
    k_vol_sums<<<nc, kVolSumThreads, 0, st>>>(P, vm, emol2, eabs2, esum, esum_abs, act, 4);
    k_vol_decide<<<(nc + 127) / 128, 128, 0, st>>>(P, vm, esum, esum_abs, trace, trace_slot,
                                                  trace_stride, act, nc, 1);
    k_vol_list<<<1, 32, 0, st>>>(P, vm, act, nc, 5, vlist);
    k_vol_pair_sums_list<<<grid, kVolThreads, 0, st>>>(P, mol_chain, vm, vlist, nc, emol2);
    k_vol_sums<<<nc, kVolSumThreads, 0, st>>>(P, vm, emol2, eabs2, esum, esum_abs, act, 5);
    k_vol_decide<<<(nc + 127) / 128, 128, 0, st>>>(P, vm, esum, esum_abs, trace, trace_slot,
                                                  trace_stride, act, nc, 2);
  }
  if (items > 0) k_vol_refresh<<<(items + 127) / 128, 128, 0, st>>>(P, mol_chain, vm, items, act);
  return cudaGetLastError();
}

}  // namespace mcgpu
