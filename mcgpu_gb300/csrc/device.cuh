// device.cuh -- device-side layout and building blocks of the GB300 trial-move
// energy path.
//
// HBM layout (one "pool" holds one box or many chains, all rows
// pool-absolute):
//   atoms      x,y,z,sig,eps,q   FP64 master rows (the SimBox rows,
//                                SimBox.h:120-149) -- moves and the FP64
//                                path read these
//              aoff  float4      (x,y,z) - anchor, FP32, w = sigma (0 for a
//                                dummy site); anchor = first primary atom
//              aeq   float2      (2*sqrt|eps|, q*sqrt(332.06)), 0 for dummies
//   molecules  mstart,mlen       MOL_START / MOL_LEN
//              mpi   int2        (MOL_PIDX_START, MOL_PIDX_COUNT)
//              mfix  uint4       anchor position in 32-bit fixed point of the
//                                box edge: differences wrap to the minimum
//                                image for free and convert with one I2F
//              mrad  float       max |atom - anchor| (rigid: move-invariant)
//              mlen packs (atoms | non-dummy atoms << 8)
//   primaries  pidx              primaryIndexes, absolute
//              ppos  float4      primary position wrapped into [0, L), FP32,
//                                for the cutoff screen
//   chains     hdr   ChainHdr    per-chain offsets, box, RNG key, counters
//
// The cutoff decision is the reference's FP64 test (SimulationStep.cpp:
// 317-330): the FP32 screen decides outright only outside a guard band
// around rc^2 and re-tests in FP64 from the master rows inside it.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/mcgpu_gb300.h"

namespace mcgpu {

constexpr int kMaxA = MCGPU_MAX_MOL_ATOMS;
constexpr int kMaxP = MCGPU_MAX_MOL_PIDX;
constexpr double kBoltz = 0.00198717;        // SimBox.h:16
constexpr double kCoulomb = 332.06;          // SimulationStep.cpp:364
// 1 atm in kcal/mol/A^3: 101325 Pa * 1e-30 m^3/A^3 * N_A / 4184 J/kcal.
constexpr double kAtmKcal = 1.4583972574259083e-05;
// Bound on the FP32-pair rounding error of a molecule energy, relative to
// the sum of the magnitudes of its FP32 terms (observed worst case ~1e-8;
// the bound keeps a 100x margin).
constexpr double kTieRel = 1e-6;
// The same for double-float pair terms (about 1e-13 observed; the bound
// keeps a 1000x margin).
constexpr double kDfRel = 1e-10;

// Device error status words (ChainHdr::error, Pool::error).
enum : int {
  kErrNone = 0,
  kErrListOverflow = 1,
  kErrBadIndex = 2,
  kErrNonFinite = 3,
  kErrWindowSync = 4,   // a cluster-wide wait of the windowed chain kernel ran out
};

// Per-chain header, one per chain (a single box is chain 0).
struct __align__(16) ChainHdr {
  int atom0, mol0, pidx0, n_mol;      // pool offsets and molecule count
  int n_atom, n_pidx, max_len, tpm;   // tpm: lanes per neighbour molecule
  int rot_mode, chain_id, simple_prim, precise;  // simple_prim: one primary per molecule;
                                                  // precise: compensated displacements
  float Lf[3], cut2_lo;               // FP32 box and guard band
  float fxs[3], cut2_hi;              // fixed point -> Angstrom scale
  float fxinvf[3], kTinvf;            // Angstrom -> fixed point (FP32); 1/kT (FP32)
  float fxs_lo[3], rad_max;           // fxs + fxs_lo = L / 2^32 to ~48 bits;
                                      // rad_max: largest molecule radius
  double L[3], cutoff;
  double fxinv[3], kT;                // Angstrom -> fixed point scale
  double max_t, max_r, energy;
  double lrc_v;                       // long-range LJ correction x volume (NPT term)
  unsigned long long seed, step;
  long long accepted, pairs;
  int error, ties, fp64_pairs, win_redo;  // ties: steps evaluated with FP64 pairs;
                                          // fp64_pairs: every step with FP64 pairs;
                                          // win_redo: steps of a window (windowed chain
                                          // kernel) re-evaluated after earlier steps
  // isobaric (NPT) volume moves: every vol_interval steps (0 = NVT), ln V
  // step uniform in +-max_dlnv, pressure in kcal/mol/A^3
  double pressure, max_dlnv;
  int vol_interval, vol_tried, vol_accepted, pad6;
  // step_limit > 0 stops the chain there (a served job's length);
  // vol_step: step count of the last volume move (one per step count)
  long long step_limit, vol_step;
  // Verlet list: nl_on enables it; nl_valid while every molecule's
  // primaries are within skin/2 of their positions at the last build;
  // cells: ncell[k] cells per edge from cell0 in the pool's cell arrays
  // (at most cell_cap); nl_r2: list radius squared; nl_half2: (skin/2)^2
  int nl_on, nl_valid, nl_builds, nl_full;
  int cell0, cell_cap, ncell[3];
  int nl_overflow;
  float nl_r2, nl_half2, nl_rlist, prad;
  int vol_mixed;        // volume moves with FP32 pairs (FP64 re-take near threshold)
  int vol_fp64;         // volume decisions re-taken with FP64 pairs
  int vncell[3];        // cells per edge of the volume move in flight
  int pad8;
  // uniform chain: one species (every molecule ulen atoms, uact active, the
  // same parameters slot by slot) laid out contiguously from atom0, one
  // primary at slot uprim, radius <= umrad: atom and primary indexes and
  // pair factors follow from the molecule index (no loads)
  int uniform, ulen, uact, uprim;
  float umrad;
  unsigned ljmask;      // uniform chains of <= 4 atoms: bits 4k + i set where the LJ term
                        // of atoms i and k is not exactly zero (set by the step kernel)
  float pad10, pad11;
  // bound on |energy - FP64 system energy of the current state|: the sum of
  // the FP32 step bounds since the energy was last set from a fresh total
  double run_err, pad12;
};
static_assert(sizeof(ChainHdr) % 16 == 0, "ChainHdr alignment");

// Guard band of the FP32 cutoff screen around rc^2 for box edges up to
// Lmax: FP32 positions carry ~1.5 ulp(Lmax) each, r2 adds its own rounding.
__host__ __device__ inline double screen_band(double rc, double Lmax) {
  int ex = 0;
  frexp(Lmax, &ex);                         // Lmax in [2^(ex-1), 2^ex)
  const double ulpL = ldexp(1.0, ex - 1 - 23);
  return 4.0 * (2.0 * 1.7320508075688772 * rc * 1.5 * ulpL + 4.0 * ldexp(rc * rc, -24)) + 1e-6;
}

// Box-derived header fields (FP32 box, fixed-point scales, screen band) for
// edges L; the same code runs at upload and after an accepted volume move.
__host__ __device__ inline void hdr_set_box(ChainHdr& h, const double L[3]) {
  double Lmax = 0;
  for (int k = 0; k < 3; k++) {
    h.L[k] = L[k];
    h.Lf[k] = (float)L[k];
    h.fxinv[k] = 4294967296.0 / L[k];
    h.fxs[k] = (float)(L[k] / 4294967296.0);
    h.fxinvf[k] = (float)(4294967296.0 / L[k]);
    h.fxs_lo[k] = (float)(L[k] / 4294967296.0 - (double)h.fxs[k]);
    Lmax = L[k] > Lmax ? L[k] : Lmax;
  }
  const double band = screen_band(h.cutoff, Lmax);
  h.cut2_lo = (float)(h.cutoff * h.cutoff - band);
  h.cut2_hi = (float)(h.cutoff * h.cutoff + band);
}

// Verlet-list configuration of one chain (host-computed).
struct NlCfg {
  int on, cell0, cell_cap, pad;
  float r2, half2, rlist, pad2;
};

// Box-derived FP32 scales of one of the two volumes of a move.
struct VolBox {
  float Lf[3], fxs[3], fxs_lo[3];
  float cut2_lo, cut2_hi;
  double L[3];
};

// One chain's volume move in flight (NPT), with both volumes' FP32 scales
// and the anchor reach of the pair screen (set once per move).
struct VolMove {
  VolBox box[2];
  float reach, sf;   // rc + 2 prad + 0.01; edge ratio L'/L
  double L[3];
  double dlnv, u;
  int state;   // 0 not due, 1 evaluate, 2 rejected outright, 3 accepted;
               // too close to the threshold: 6 after the FP32 U(V'), re-take
               // U(V') in double-float; 4 after that, re-take both totals in
               // double-float; 5 after that, re-take both in FP64
  int fp64;    // decided on FP64 pair energies
};

// Molecules a volume phase covers: all of the pool (act == nullptr) or the
// ranges [act_m0[k], act_m0[k] + act_pref[k+1] - act_pref[k]) of n_act
// active chains, act_pref their prefix sums (device arrays).
struct MolRanges {
  const int* act_slot = nullptr;   // chain (slot) of each active range
  const int* act_m0 = nullptr;
  const int* act_pref = nullptr;
  int n_act = 0;
  int total = 0;
};

struct Pool {
  double *x, *y, *z, *sig, *eps, *q;
  float4* aoff;
  float4* aofl;        // plain path: low part of the offsets (FP64 offset - aoff)
  double2* blend;      // FP64 blending factors (sqrt sigma, sqrt eps; -1 for a skipped
                       // site), or null (pools of the served form)
  float2* aeq;
  int *mstart, *mlen;
  int2* mpi;
  uint4* mfix;
  float* mrad;
  float4* mq;          // device-resident chains: unit quaternion (w, x, y, z)
  float4* atpl;        // device-resident chains: template offsets R(q)^-1 o
  int* pidx;
  float4* ppos;
  ChainHdr* hdr;
  double* rb;          // rollback rows, 3 * max_len per chain
  mcgpu_trace* trace;  // optional step records
  int n_chains;
  // Verlet lists (null when no chain uses one)
  int* nl;             // [n_mol * nl_stride] neighbour molecules (pool-absolute)
  int* nl_cnt;         // [n_mol]
  float4* pbuild;      // [n_pidx] primary screen positions at the last build
  int* mcell;          // [n_mol] cell of each molecule (pool cell index)
  int* cell_cnt;       // [cells] members, then fill counters
  int* cell_start;     // [cells] first slot in cell_mol
  int* cell_mol;       // [n_mol] molecules grouped by cell
  int nl_stride;
  // cell grid of a volume move, indexed in the chain's own molecule range
  // (a chain has at most as many cells as molecules); null without NPT
  int* vc_cnt;         // [n_mol] members of cell mol0 + c
  int* vc_start;       // [n_mol] first slot in vc_mol
  int* vc_mol;         // [n_mol] molecules grouped by cell
  int* vc_of;          // [n_mol] cell of each molecule
};

// ---- Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), from the published
// description: ten rounds, two 32x32->64 multiplies per round, Weyl key bumps.
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    unsigned hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    unsigned hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += 0x9E3779B9u;
    k.y += 0xBB67AE85u;
  }
  return c;
}
__device__ __forceinline__ double u01(unsigned r) {
  return ((double)r + 0.5) * 2.3283064365386963e-10;
}
__device__ __forceinline__ int uidx(unsigned r, int n) {
  return (int)(((unsigned long long)r * (unsigned long long)n) >> 32);
}

// A trial move: vertex, translation, rotation (Euler degrees or axis+angle).
struct Proposal {
  int mol, vertex, mode, trig;   // trig: cos/sin below hold the Euler angles' values
  double dx, dy, dz, r0, r1, r2, r3, u;
  double cs[3], sn[3];           // host-drawn Euler moves: cos, sin of each angle
};

// Draws the proposal of (seed, chain, step): the counter layout and the
// uniform/index mappings are fixed so a CPU replay gets the same values.
__device__ inline Proposal draw_proposal(unsigned long long seed, unsigned chain,
                                         unsigned long long step, int n_mol,
                                         const int* mlen_chain, double max_t,
                                         double max_r, int mode) {
  uint2 key = make_uint2((unsigned)seed, (unsigned)(seed >> 32));
  uint4 a = philox4x32_10(make_uint4((unsigned)step, (unsigned)(step >> 32), chain, 0u), key);
  uint4 c = philox4x32_10(make_uint4((unsigned)step, (unsigned)(step >> 32), chain, 1u), key);
  uint4 d = philox4x32_10(make_uint4((unsigned)step, (unsigned)(step >> 32), chain, 2u), key);
  Proposal p;
  p.mol = uidx(a.x, n_mol);
  p.vertex = uidx(a.y, mlen_chain[p.mol] & 255);
  p.mode = mode;
  p.trig = 0;
  p.dx = __dadd_rn(__dmul_rn(2.0 * max_t, u01(a.z)), -max_t);
  p.dy = __dadd_rn(__dmul_rn(2.0 * max_t, u01(a.w)), -max_t);
  p.dz = __dadd_rn(__dmul_rn(2.0 * max_t, u01(c.x)), -max_t);
  if (mode == MCGPU_ROT_EULER) {
    p.r0 = __dadd_rn(__dmul_rn(2.0 * max_r, u01(c.y)), -max_r);
    p.r1 = __dadd_rn(__dmul_rn(2.0 * max_r, u01(c.z)), -max_r);
    p.r2 = __dadd_rn(__dmul_rn(2.0 * max_r, u01(c.w)), -max_r);
    p.r3 = 0.0;
  } else {
    double zc = __dadd_rn(__dmul_rn(2.0, u01(c.y)), -1.0);
    double phi = __dmul_rn(6.283185307179586, u01(c.z));
    double s = sqrt(__dadd_rn(1.0, -__dmul_rn(zc, zc)));
    double sp, cp;
    sincos(phi, &sp, &cp);
    p.r0 = __dmul_rn(s, cp);
    p.r1 = __dmul_rn(s, sp);
    p.r2 = zc;
    p.r3 = __dadd_rn(__dmul_rn(2.0 * max_r, u01(c.w)), -max_r);
  }
  p.u = u01(d.x);
  return p;
}

// Rotation matrix of a proposal, applied to v = atom - pivot:
// Euler: rotateX, then rotateY, then rotateZ (SimulationStep.cpp:400-422),
// composed as separate rounded steps exactly like the reference.
struct Rot {
  double cx, sx, cy, sy, cz, sz;   // Euler; axis form: cx=cos, sx=sin, cy=1-cos
  double kx, ky, kz;               // axis form: unit axis
  int mode;
};

__device__ inline Rot make_rot(const Proposal& p) {
  Rot R;
  R.mode = p.mode;
  if (p.mode == MCGPU_ROT_EULER && p.trig) {
    R.cx = p.cs[0]; R.sx = p.sn[0];
    R.cy = p.cs[1]; R.sy = p.sn[1];
    R.cz = p.cs[2]; R.sz = p.sn[2];
  } else if (p.mode == MCGPU_ROT_EULER) {
    sincos(__dmul_rn(p.r0, 3.14159265358979) / 180.0, &R.sx, &R.cx);
    sincos(__dmul_rn(p.r1, 3.14159265358979) / 180.0, &R.sy, &R.cy);
    sincos(__dmul_rn(p.r2, 3.14159265358979) / 180.0, &R.sz, &R.cz);
  } else {
    sincos(__dmul_rn(p.r3, 3.14159265358979) / 180.0, &R.sx, &R.cx);
    R.cy = __dadd_rn(1.0, -R.cx);
    R.kx = p.r0; R.ky = p.r1; R.kz = p.r2;
  }
  return R;
}

// Applies the rotation to v (in place).
__device__ __forceinline__ void rot_apply(const Rot& R, double& vx, double& vy, double& vz) {
  if (R.mode == MCGPU_ROT_EULER) {
    double oy = vy, oz = vz;   // rotateX
    vy = __dadd_rn(__dmul_rn(oy, R.cx), __dmul_rn(oz, R.sx));
    vz = __dadd_rn(__dmul_rn(oz, R.cx), -__dmul_rn(oy, R.sx));
    oz = vz;
    double ox = vx;            // rotateY
    vz = __dadd_rn(__dmul_rn(oz, R.cy), __dmul_rn(ox, R.sy));
    vx = __dadd_rn(__dmul_rn(ox, R.cy), -__dmul_rn(oz, R.sy));
    ox = vx;
    oy = vy;                   // rotateZ
    vx = __dadd_rn(__dmul_rn(ox, R.cz), __dmul_rn(oy, R.sz));
    vy = __dadd_rn(__dmul_rn(oy, R.cz), -__dmul_rn(ox, R.sz));
  } else {
    // Rodrigues: v' = v c + (k x v) s + k (k.v)(1-c)
    double kv = R.kx * vx + R.ky * vy + R.kz * vz;
    double qx = R.ky * vz - R.kz * vy, qy = R.kz * vx - R.kx * vz, qz = R.kx * vy - R.ky * vx;
    double x = vx * R.cx + qx * R.sx + R.kx * kv * R.cy;
    double y = vy * R.cx + qy * R.sx + R.ky * kv * R.cy;
    double z = vz * R.cx + qz * R.sx + R.kz * kv * R.cy;
    vx = x; vy = y; vz = z;
  }
}

// SimCalcs::makePeriodic (SimulationStep.cpp:377-385), FP64.
__device__ __forceinline__ double make_periodic(double x, double L) {
  if (x < -0.5 * L) x = __dadd_rn(x, L);
  if (x > 0.5 * L) x = __dadd_rn(x, -L);
  return x;
}

// Double-float accumulation: (hi, lo) += v with Knuth's two-sum, so sums of
// FP32 terms keep ~48 significant bits without FP64 instructions.
__device__ __forceinline__ void ff_add(float& hi, float& lo, float v) {
  const float s = __fadd_rn(hi, v);
  const float bb = __fsub_rn(s, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(v, bb));
  hi = s;
  lo = __fadd_rn(lo, err);
}

// (hi, lo) += (h2, l2).
__device__ __forceinline__ void ff_add2(float& hi, float& lo, float h2, float l2) {
  ff_add(hi, lo, h2);
  lo = __fadd_rn(lo, l2);
}

// Exact int -> float for |x| < 2^22 by integer arithmetic on the bits of
// 1.5 * 2^23 (no conversion instruction: on this part those issue on the
// slow FP64 pipe).
__device__ __forceinline__ float small_i2f(int x) {
  return __int_as_float(0x4B400000 + x) - 12582912.0f;
}

// ---- double-float arithmetic ----------------------------------------------
// A value h + l with |l| <= ulp(h)/2 (about 48 significant bits) on FP32
// instructions: Knuth's two-sum, the FMA two-product, and the usual
// renormalised sum and product (Dekker 1971; Hida, Li, Bailey 2001).
// Relative error of an operation about 2^-44.
struct df {
  float h, l;
};

__device__ __forceinline__ df df_of(double x) {
  const float h = __double2float_rn(x);
  return {h, __double2float_rn(x - (double)h)};
}
__device__ __forceinline__ df df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ df df_quick(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ df df_add(df a, df b) {
  df s = df_two_sum(a.h, b.h);
  const df t = df_two_sum(a.l, b.l);
  s = df_quick(s.h, __fadd_rn(s.l, t.h));
  return df_quick(s.h, __fadd_rn(s.l, t.l));
}
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, {-b.h, -b.l}); }
__device__ __forceinline__ df df_mul(df a, df b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  return df_quick(p, e);
}
// 1/sqrt(a) for a > 0: an FP32 estimate refined by one Newton step
// y + (y/2)(1 - a y^2) in double-float (error ~1e-14 relative).
__device__ __forceinline__ df df_rsqrt(df a) {
  const float y = rsqrtf(a.h);
  const float y2 = __fmul_rn(y, y);
  const df ay2 = df_mul(a, {y2, fmaf(y, y, -y2)});
  const df r = df_sub({1.0f, 0.0f}, ay2);
  return df_add({y, 0.0f}, df_mul(r, {0.5f * y, 0.0f}));
}

// ---- groups: the warps that advance one chain --------------------------
struct Group {
  int tid, nthreads, bar;
  __device__ __forceinline__ int warp() const { return tid >> 5; }
  __device__ __forceinline__ int nwarps() const { return nthreads >> 5; }
  __device__ __forceinline__ void sync() const {
    if (nthreads == 32) {
      __syncwarp();
    } else {
      asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(nthreads) : "memory");
    }
  }
};

// Shared-memory state of one group; carved from dynamic shared memory with
// sizes fixed per launch (max molecule length, warps per group).  Each warp
// owns a 64-entry ring of neighbour-list entries: the warp screens 32
// candidates per round, appends the in-range ones, and evaluates full
// batches of 32 entries, so the screen -> list -> pair pipeline needs no
// group barrier.
constexpr int kRing = 64;
// Bytes of one drawn move in shared memory (MoveF, move_f32.cuh).
constexpr int kPropBytes = 40;

struct GroupSmem {
  // moved molecule
  double* ox; double* oy; double* oz;   // old FP64 coords [maxA]
  double* nx; double* ny; double* nz;   // new FP64 coords [maxA]
  double* sd; double* ed; double* qd;   // FP64 sigma, epsilon, charge [maxA]
  float4* o_old; float4* o_new;         // FP32 offsets from the anchor, w=sigma [maxA]
  float4* l_old; float4* l_new;         // their low parts (plain path; zero for chains) [maxA]
  float4* eq;                           // FP32 (2sqrt|eps|, q sqrt(332.06), |o_old|^2, |o_new|^2) [maxA]
  float4* p_old; float4* p_new;         // wrapped FP32 primaries [kMaxP]
  int* pa;                              // primary atom slots in the molecule [kMaxP]
  // per-warp neighbour rings [nwarps * kRing]
  int* lj;                              // (j << 4) | flags
  float4* lA;                           // (Dold.xyz, Dnew.x)
  float2* lB;                           // (Dnew.y, Dnew.z)
  double* red;                          // [2][3 * nwarps] reduction scratch (two buffers)
  long long* redl;                      // [2][nwarps]
  int* misc;                            // [32] broadcast ints
  double* miscd;                        // [32] broadcast doubles
  float4* pc;                           // [cache_n] screen positions of the chain (or null)
  void* props;                          // [32] drawn moves of the next steps (chain kernel)
  float4* nbuf;                         // [nwarps * 32 * 5] per-lane neighbour rows (async copies)
  float2* teq;                          // [maxA] pair factors per slot of a uniform chain
  char* ahead;                          // three more staging slots (the chain kernel's moves)
};

// The rows a staged move occupies: offsets, pair factors, primaries, the
// broadcast ints and doubles: the ones inside GroupSmem, and three more the
// chain kernel rotates through (a step's move, the next one staged ahead,
// and the one before, which slower warps may still be committing).
struct StageSlot {
  float4* o_old; float4* o_new;
  float4* l_old; float4* l_new;
  float4* eq;
  float4* p_old; float4* p_new;
  int* pa;
  int* misc;
  double* miscd;
};

// s with its staging rows replaced by slot t's.
__device__ __forceinline__ GroupSmem with_slot(GroupSmem s, const StageSlot& t) {
  s.o_old = t.o_old; s.o_new = t.o_new; s.l_old = t.l_old; s.l_new = t.l_new; s.eq = t.eq;
  s.p_old = t.p_old; s.p_new = t.p_new; s.pa = t.pa; s.misc = t.misc; s.miscd = t.miscd;
  return s;
}

struct SmemShape {
  int maxA, nwarps, cache_n;
  __host__ __device__ static int align16(int v) { return (v + 15) & ~15; }
  __host__ __device__ int bytes() const {
    int b = 0;
    b += align16(9 * maxA * 8);
    b += align16(4 * maxA * 16);
    b += align16(maxA * 16);
    b += align16(2 * kMaxP * 16);
    b += align16(kMaxP * 4);
    b += align16(nwarps * kRing * 4);
    b += align16(nwarps * kRing * 16);
    b += align16(nwarps * kRing * 8);
    b += align16(6 * nwarps * 8);
    b += align16(2 * nwarps * 8);
    b += align16(32 * 4);
    b += align16(32 * 8);
    b += align16(cache_n * 16);
    b += align16(32 * kPropBytes);
    b += align16(nwarps * 32 * 5 * 16);
    b += align16(maxA * 8);
    b += 3 * ahead_bytes();
    return b;
  }
  // the second staging slot: offsets and factors, primaries, misc, miscd
  __host__ __device__ int ahead_bytes() const {
    return align16(5 * maxA * 16) + align16(2 * kMaxP * 16) + align16(kMaxP * 4) + align16(32 * 4) +
           align16(32 * 8);
  }
  __device__ StageSlot ahead_slot(char* p) const {
    StageSlot t;
    t.o_old = (float4*)p; t.o_new = t.o_old + maxA; t.l_old = t.o_new + maxA;
    t.l_new = t.l_old + maxA; t.eq = t.l_new + maxA; p += align16(5 * maxA * 16);
    t.p_old = (float4*)p; t.p_new = t.p_old + kMaxP; p += align16(2 * kMaxP * 16);
    t.pa = (int*)p; p += align16(kMaxP * 4);
    t.misc = (int*)p; p += align16(32 * 4);
    t.miscd = (double*)p;
    return t;
  }
  __device__ GroupSmem carve(char* base) const {
    GroupSmem s;
    char* p = base;
    s.ox = (double*)p; s.oy = s.ox + maxA; s.oz = s.oy + maxA;
    s.nx = s.oz + maxA; s.ny = s.nx + maxA; s.nz = s.ny + maxA;
    s.sd = s.nz + maxA; s.ed = s.sd + maxA; s.qd = s.ed + maxA;
    p += align16(9 * maxA * 8);
    s.o_old = (float4*)p; s.o_new = s.o_old + maxA;
    s.l_old = s.o_new + maxA; s.l_new = s.l_old + maxA; p += align16(4 * maxA * 16);
    s.eq = (float4*)p; p += align16(maxA * 16);
    s.p_old = (float4*)p; s.p_new = s.p_old + kMaxP; p += align16(2 * kMaxP * 16);
    s.pa = (int*)p; p += align16(kMaxP * 4);
    s.lj = (int*)p; p += align16(nwarps * kRing * 4);
    s.lA = (float4*)p; p += align16(nwarps * kRing * 16);
    s.lB = (float2*)p; p += align16(nwarps * kRing * 8);
    s.red = (double*)p; p += align16(6 * nwarps * 8);
    s.redl = (long long*)p; p += align16(2 * nwarps * 8);
    s.misc = (int*)p; p += align16(32 * 4);
    s.miscd = (double*)p; p += align16(32 * 8);
    s.pc = cache_n > 0 ? (float4*)p : nullptr;
    p += align16(cache_n * 16);
    s.props = (void*)p;
    p += align16(32 * kPropBytes);
    s.nbuf = (float4*)p;
    p += align16(nwarps * 32 * 5 * 16);
    s.teq = (float2*)p;
    p += align16(maxA * 8);
    s.ahead = p;
    return s;
  }
};

// Flags of a neighbour-list entry.
enum : int { kInOld = 1, kInNew = 2, kWrapOld = 4, kWrapNew = 8 };

// Moved-molecule scalars, identical in every thread of a group after
// staging.  states: bit 0 = evaluate the current ("old") placement, bit 1 =
// evaluate the proposed ("new") placement.
struct MovedInfo {
  int mol, atom0, len, npidx, act, states, vertex, pad;
  uint4 fx_old, fx_new;
  float rad, qm;  // qm: net FP32 charge factor sum_a q_a sqrt(332.06)
};

__device__ __forceinline__ float wrapf(float d, float L) {
  float a = fabsf(d);
  return fminf(a, L - a);
}

// Reciprocal square root, hardware estimate refined by one Newton-Raphson
// step y' = y + (y/2)(1 - r2 y^2): the estimate is good to about 2^-23
// relative, the refined value to about one ulp.
__device__ __forceinline__ float rsqrt_nr(float r2) {
  float ir = rsqrtf(r2);
  const float t0 = r2 * ir;
  const float h = fmaf(-t0, ir, 1.0f);
  return fmaf(0.5f * ir, h, ir);
}

// Hardware reciprocal estimate (rcp.approx, ~1 ulp); used only on a factor
// of an already small term, where its relative error is harmless.
__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// 1/r2 to about one ulp: hardware reciprocal estimate refined by one
// Newton-Raphson step y' = y (2 - r2 y).
__device__ __forceinline__ float rcp_nr(float r2) {
  const float y = rcp_approx(r2);
  return y * fmaf(-r2, y, 2.0f);
}

// LJ part of a pair term from per-atom factors (sigma, 2sqrt|eps|) and
// 1/r2: 4 eps (s^12 - s^6), s = sigma_ab^2 / r^2 with geometric blending
// (SimulationStep.cpp:344-358, :369-375).  The r^-12 term amplifies the
// relative error of s twelvefold, so s is formed from a refined 1/r2 (one
// rounding) rather than from (1/r)^2.
__device__ __forceinline__ float lj32(float ir2, float sa, float sb, float ea, float eb) {
  const float t = (sa * sb) * ir2;
  const float t3 = t * t * t;
  return (ea * eb) * fmaf(t3, t3, -t3);
}

// FP64 pair term restating SimulationStep.cpp:344-375 and
// BruteForceStep.cpp:64-73 for a non-dummy pair at squared distance r2.
// FP64 pair term of the reference (SimCalcs::calcLJEnergy / calcChargeEnergy
// with BruteForceStep's blending, SimulationStep.cpp:344-375) from the
// blending factors sa = sqrt(sigma_a), sb = sqrt(sigma_b), ea = sqrt(eps_a),
// eb = sqrt(eps_b) and 1/r from one FP64 rsqrt: sigma_ab^2 = (sa sb)^2,
// eps_ab = ea eb.  Each term is within a few ulps of the reference's (two
// square roots, a square root and two divisions per pair cost many passes
// of GB300's FP64 pipe); sums differ from the reference's at the FP64
// rounding of their order.
__device__ __forceinline__ double pair64(double r2, double sa, double sb, double ea, double eb,
                                         double qa, double qb) {
  if (r2 == 0.0) return 0.0;
  const double ri = rsqrt(r2);
  const double sig = sa * sb;
  const double s2r2 = (sig * sig) * (ri * ri);
  const double s6r6 = s2r2 * s2r2 * s2r2;
  const double lj = 4.0 * (ea * eb) * (s6r6 * s6r6 - s6r6);
  return lj + (qa * qb * kCoulomb) * ri;
}

// The blending factor rows of an atom for pair64: sqrt(sigma) and
// sqrt(eps); sigma = -1 marks a site the reference skips (a negative sigma
// or epsilon, BruteForceStep.cpp:64-65).
__device__ __forceinline__ double2 blend64(double sig, double eps) {
  if (!(sig >= 0 && eps >= 0)) return make_double2(-1.0, 0.0);
  return make_double2(sqrt(sig), sqrt(eps));
}

}  // namespace mcgpu
