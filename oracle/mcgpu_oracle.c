/*
 * mcgpu_oracle.c -- CPU FP64 restatement of MCGPU's Metropolis trial-move
 * energy path.  TEST INFRASTRUCTURE ONLY (the checker and the timed CPU
 * baseline); the product never links or calls this file.
 *
 * Reference files are cited by their path inside the MCGPU project.  The
 * arithmetic (operation order, pow/sqrt/cos/sin/exp calls, summation order)
 * follows the reference line by line so that results are bit-identical to the
 * reference compiled with g++ on the same machine; the file must be built with
 * -ffp-contract=off so that no compiler fuses a*b+c where the reference does
 * not (aarch64 gcc fuses by default).
 */
#include "mcgpu_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ---- pair math ---------------------------------------------------------- */

/* SimCalcs::makePeriodic, src/Metropolis/SimulationStep.cpp:377-385:
 * single-image minimum image, "+L if below -L/2" then "-L if above +L/2". */
double orc_make_periodic(double x, double dim_len) {
  int lt = (x < -0.5 * dim_len);
  x += lt * dim_len;
  int gt = (x > 0.5 * dim_len);
  x -= gt * dim_len;
  return x;
}

/* SimCalcs::calcAtomDistSquared, src/Metropolis/SimulationStep.cpp:332-342
 * (difference taken as a2 - a1). */
double orc_atom_dist2(const orc_box* b, int a1, int a2) {
  double dx = orc_make_periodic(b->x[a2] - b->x[a1], b->size[0]);
  double dy = orc_make_periodic(b->y[a2] - b->y[a1], b->size[1]);
  double dz = orc_make_periodic(b->z[a2] - b->z[a1], b->size[2]);
  return dx * dx + dy * dy + dz * dz;
}

/* SimCalcs::calcBlending, src/Metropolis/SimulationStep.cpp:369-375. */
double orc_blend(double a, double c) {
  if (a * c >= 0) return sqrt(a * c);
  return sqrt(-1 * a * c);
}

/* SimCalcs::calcLJEnergy, src/Metropolis/SimulationStep.cpp:344-358. */
double orc_lj(const orc_box* b, int a1, int a2, double r2) {
  if (r2 == 0.0) return 0.0;
  const double sigma = orc_blend(b->sigma[a1], b->sigma[a2]);
  const double epsilon = orc_blend(b->epsilon[a1], b->epsilon[a2]);
  const double s2r2 = pow(sigma, 2) / r2;
  const double s6r6 = pow(s2r2, 3);
  const double s12r12 = pow(s6r6, 2);
  return 4.0 * epsilon * (s12r12 - s6r6);
}

/* SimCalcs::calcChargeEnergy, src/Metropolis/SimulationStep.cpp:360-367. */
double orc_charge(const orc_box* b, int a1, int a2, double r) {
  if (r == 0.0) return 0.0;
  const double e = 332.06;
  return (b->charge[a1] * b->charge[a2] * e) / r;
}

/* SimCalcs::moleculesInRange, src/Metropolis/SimulationStep.cpp:317-330:
 * true when ANY primary-index pair is within the cutoff (inclusive). */
int orc_molecules_in_range(const orc_box* b, int p1s, int p1e, int p2s, int p2e) {
  int out = 0;
  for (int p1i = p1s; p1i < p1e; p1i++) {
    int p1 = b->pidx[p1i];
    for (int p2i = p2s; p2i < p2e; p2i++) {
      int p2 = b->pidx[p2i];
      out |= (orc_atom_dist2(b, p1, p2) <= b->cutoff * b->cutoff);
    }
  }
  return out;
}

/* BruteForceCalcs::calcMoleculeInteractionEnergy,
 * src/Metropolis/BruteForceStep.cpp:48-79.  Atoms with sigma<0 or epsilon<0
 * (dummy sites) are skipped; coincident atoms contribute 0. */
double orc_mol_pair_energy(const orc_box* b, int m1, int m2) {
  double sum = 0;
  const int s1 = b->mol_start[m1], e1 = s1 + b->mol_len[m1];
  const int s2 = b->mol_start[m2], e2 = s2 + b->mol_len[m2];
  for (int i = s1; i < e1; i++) {
    for (int j = s2; j < e2; j++) {
      if (b->sigma[i] >= 0 && b->sigma[j] >= 0 && b->epsilon[i] >= 0 &&
          b->epsilon[j] >= 0) {
        const double r2 = orc_atom_dist2(b, i, j);
        if (r2 == 0.0) {
          sum += 0.0;
        } else {
          sum += orc_lj(b, i, j, r2);
          sum += orc_charge(b, i, j, sqrt(r2));
        }
      }
    }
  }
  return sum;
}

/* BruteForceCalcs::calcMolecularEnergyContribution,
 * src/Metropolis/BruteForceStep.cpp:15-46: sum over otherMol in
 * [startMol, N), otherMol != currMol, of the pair energy of in-range
 * molecules, accumulated in increasing otherMol order. */
double orc_mol_energy(const orc_box* b, int curr, int start) {
  double total = 0;
  const int p1s = b->mol_pidx_start[curr];
  const int p1e = b->mol_pidx_count[curr] + p1s;
  for (int other = start; other < b->n_mol; other++) {
    if (other != curr) {
      int p2s = b->mol_pidx_start[other];
      int p2e = b->mol_pidx_count[other] + p2s;
      if (orc_molecules_in_range(b, p1s, p1e, p2s, p2e))
        total += orc_mol_pair_energy(b, curr, other);
    }
  }
  return total;
}

/* Sum of the magnitudes of the terms orc_mol_energy adds (per atom pair:
 * 4 eps s^12, 4 eps s^6 and |Coulomb|): the scale of the cancellation in a
 * molecule energy, used to set the tolerance of FP32-pair results
 * (|err| <= 1e-5 * max(|E|, 1e-3 * this)). */
double orc_mol_energy_abs(const orc_box* b, int curr, int start) {
  double total = 0;
  const int p1s = b->mol_pidx_start[curr];
  const int p1e = b->mol_pidx_count[curr] + p1s;
  for (int other = start; other < b->n_mol; other++) {
    if (other == curr) continue;
    int p2s = b->mol_pidx_start[other];
    int p2e = b->mol_pidx_count[other] + p2s;
    if (!orc_molecules_in_range(b, p1s, p1e, p2s, p2e)) continue;
    const int s1 = b->mol_start[curr], e1 = s1 + b->mol_len[curr];
    const int s2 = b->mol_start[other], e2 = s2 + b->mol_len[other];
    for (int i = s1; i < e1; i++)
      for (int j = s2; j < e2; j++) {
        if (!(b->sigma[i] >= 0 && b->sigma[j] >= 0 && b->epsilon[i] >= 0 && b->epsilon[j] >= 0))
          continue;
        const double r2 = orc_atom_dist2(b, i, j);
        if (r2 == 0.0) continue;
        /* the three terms of the pair energy: 4 eps s^12, -4 eps s^6, Coulomb */
        const double sig = orc_blend(b->sigma[i], b->sigma[j]);
        const double eps = orc_blend(b->epsilon[i], b->epsilon[j]);
        const double s6 = pow(pow(sig, 2) / r2, 3);
        total += 4.0 * eps * s6 * s6 + 4.0 * eps * s6 + fabs(orc_charge(b, i, j, sqrt(r2)));
      }
  }
  return total;
}

/* Like orc_mol_energy_abs with each term weighted by its condition number
 * with respect to the pair distance, |d ln t / d ln r|: 12 for 4 eps s^12,
 * 6 for 4 eps s^6, 1 for Coulomb.  A term evaluated from positions with
 * relative error d carries an error of about (weight * |t| * d), so this
 * sum sets the rounding scale of FP32 pair terms at close contacts. */
double orc_mol_energy_absk(const orc_box* b, int curr, int start) {
  double total = 0;
  const int p1s = b->mol_pidx_start[curr];
  const int p1e = b->mol_pidx_count[curr] + p1s;
  for (int other = start; other < b->n_mol; other++) {
    if (other == curr) continue;
    int p2s = b->mol_pidx_start[other];
    int p2e = b->mol_pidx_count[other] + p2s;
    if (!orc_molecules_in_range(b, p1s, p1e, p2s, p2e)) continue;
    const int s1 = b->mol_start[curr], e1 = s1 + b->mol_len[curr];
    const int s2 = b->mol_start[other], e2 = s2 + b->mol_len[other];
    for (int i = s1; i < e1; i++)
      for (int j = s2; j < e2; j++) {
        if (!(b->sigma[i] >= 0 && b->sigma[j] >= 0 && b->epsilon[i] >= 0 && b->epsilon[j] >= 0))
          continue;
        const double r2 = orc_atom_dist2(b, i, j);
        if (r2 == 0.0) continue;
        const double sig = orc_blend(b->sigma[i], b->sigma[j]);
        const double eps = orc_blend(b->epsilon[i], b->epsilon[j]);
        const double s6 = pow(pow(sig, 2) / r2, 3);
        total += 12.0 * 4.0 * eps * s6 * s6 + 6.0 * 4.0 * eps * s6 +
                 fabs(orc_charge(b, i, j, sqrt(r2)));
      }
  }
  return total;
}

/* SimulationStep::calcSystemEnergy, src/Metropolis/SimulationStep.cpp:40-71
 * with subLJ = subCharge = 0 and the intramolecular term disabled
 * (ENABLE_INTRA false, SimulationStep.h:15): sum over mol of
 * calcMoleculeEnergy(mol, mol), i.e. every in-range pair counted once. */
double orc_system_energy(const orc_box* b) {
  double total = 0;
  for (int mol = 0; mol < b->n_mol; mol++) total += orc_mol_energy(b, mol, mol);
  return total;
}

/* Counts, for molecule curr against all others, the in-range molecule pairs
 * and the atom pairs the pair loop evaluates (both atoms non-dummy).  Used to
 * fix the algorithmic work per move (F_pair per atom pair). */
int orc_count_pairs(const orc_box* b, int curr, long long* mol_pairs,
                    long long* atom_pairs) {
  const int p1s = b->mol_pidx_start[curr];
  const int p1e = b->mol_pidx_count[curr] + p1s;
  long long mp = 0, ap = 0;
  for (int other = 0; other < b->n_mol; other++) {
    if (other == curr) continue;
    int p2s = b->mol_pidx_start[other];
    int p2e = b->mol_pidx_count[other] + p2s;
    if (!orc_molecules_in_range(b, p1s, p1e, p2s, p2e)) continue;
    mp++;
    const int s1 = b->mol_start[curr], e1 = s1 + b->mol_len[curr];
    const int s2 = b->mol_start[other], e2 = s2 + b->mol_len[other];
    for (int i = s1; i < e1; i++)
      for (int j = s2; j < e2; j++)
        if (b->sigma[i] >= 0 && b->sigma[j] >= 0 && b->epsilon[i] >= 0 &&
            b->epsilon[j] >= 0)
          ap++;
  }
  *mol_pairs = mp;
  *atom_pairs = ap;
  return 0;
}

/* ---- moves -------------------------------------------------------------- */

/* SimCalcs::translateAtom, src/Metropolis/SimulationStep.cpp:703-708. */
static void translate_atom(orc_box* b, int a, double dx, double dy, double dz) {
  b->x[a] += dx;
  b->y[a] += dy;
  b->z[a] += dz;
}

/* SimCalcs::rotateX/Y/Z, src/Metropolis/SimulationStep.cpp:400-422. */
static void rotate_x(orc_box* b, int a, double deg) {
  double rad = deg * 3.14159265358979 / 180.0;
  double oy = b->y[a], oz = b->z[a];
  b->y[a] = oy * cos(rad) + oz * sin(rad);
  b->z[a] = oz * cos(rad) - oy * sin(rad);
}
static void rotate_y(orc_box* b, int a, double deg) {
  double rad = deg * 3.14159265358979 / 180.0;
  double oz = b->z[a], ox = b->x[a];
  b->z[a] = oz * cos(rad) + ox * sin(rad);
  b->x[a] = ox * cos(rad) - oz * sin(rad);
}
static void rotate_z(orc_box* b, int a, double deg) {
  double rad = deg * 3.14159265358979 / 180.0;
  double ox = b->x[a], oy = b->y[a];
  b->x[a] = ox * cos(rad) + oy * sin(rad);
  b->y[a] = oy * cos(rad) - ox * sin(rad);
}

/* SimCalcs::rotateAtom, src/Metropolis/SimulationStep.cpp:387-398. */
static void rotate_atom(orc_box* b, int a, int pivot, double rx, double ry,
                        double rz) {
  double px = b->x[pivot], py = b->y[pivot], pz = b->z[pivot];
  translate_atom(b, a, -px, -py, -pz);
  rotate_x(b, a, rx);
  rotate_y(b, a, ry);
  rotate_z(b, a, rz);
  translate_atom(b, a, px, py, pz);
}

/* Rotation of atom a by `deg` degrees about the unit axis k through the
 * pivot (Rodrigues' formula, R = cI + s[k]x + (1-c)kk^T), the random-axis
 * trial move of the device-resident forms.  No reference counterpart: the
 * reference rotates only by Euler angles. */
static void rotate_atom_axis(orc_box* b, int a, int pivot, double kx, double ky,
                             double kz, double deg) {
  double rad = deg * 3.14159265358979 / 180.0;
  double c = cos(rad), s = sin(rad), t = 1.0 - c;
  double px = b->x[pivot], py = b->y[pivot], pz = b->z[pivot];
  double vx = b->x[a] - px, vy = b->y[a] - py, vz = b->z[a] - pz;
  double kv = kx * vx + ky * vy + kz * vz;
  double cx = ky * vz - kz * vy, cy = kz * vx - kx * vz, cz = kx * vy - ky * vx;
  b->x[a] = (vx * c + cx * s + kx * kv * t) + px;
  b->y[a] = (vy * c + cy * s + ky * kv * t) + py;
  b->z[a] = (vz * c + cz * s + kz * kv * t) + pz;
}

/* SimCalcs::keepMoleculeInBox, src/Metropolis/SimulationStep.cpp:710-729:
 * if the molecule's first primary atom left [0, L] in a dimension, shift the
 * whole molecule by one box length. */
void orc_keep_in_box(orc_box* b, int mol) {
  int start = b->mol_start[mol];
  int end = start + b->mol_len[mol];
  int p = b->pidx[b->mol_pidx_start[mol]];
  double* c[3] = {b->x, b->y, b->z};
  for (int d = 0; d < 3; d++) {
    if (c[d][p] < 0) {
      for (int j = start; j < end; j++) c[d][j] += b->size[d];
    } else if (c[d][p] > b->size[d]) {
      for (int j = start; j < end; j++) c[d][j] -= b->size[d];
    }
  }
}

/* Simulation::run's initial wrap of every molecule (Simulation.cpp:70-72). */
void orc_wrap_all(orc_box* b) {
  for (int m = 0; m < b->n_mol; m++) orc_keep_in_box(b, m);
}

/* SimCalcs::intermolecularMove, src/Metropolis/SimulationStep.cpp:520-566,
 * with the seven random draws supplied in *mv: save rollback coordinates,
 * rotate every non-vertex atom about the vertex and translate it, then
 * translate the vertex and wrap the molecule by its primary atom. */
void orc_apply_move(orc_box* b, const orc_move* mv) {
  int start = b->mol_start[mv->mol];
  int len = b->mol_len[mv->mol];
  int v = mv->vertex;
  for (int i = 0; i < len; i++) {
    b->rb_x[i] = b->x[start + i];
    b->rb_y[i] = b->y[start + i];
    b->rb_z[i] = b->z[start + i];
    if (i == v) continue;
    if (mv->mode == 0)
      rotate_atom(b, start + i, start + v, mv->r0, mv->r1, mv->r2);
    else
      rotate_atom_axis(b, start + i, start + v, mv->r0, mv->r1, mv->r2, mv->r3);
    translate_atom(b, start + i, mv->dx, mv->dy, mv->dz);
  }
  b->x[start + v] += mv->dx;
  b->y[start + v] += mv->dy;
  b->z[start + v] += mv->dz;
  orc_keep_in_box(b, mv->mol);
}

/* SimCalcs::rollback, src/Metropolis/SimulationStep.cpp:731-749. */
void orc_rollback(orc_box* b, int mol) {
  int start = b->mol_start[mol];
  int len = b->mol_len[mol];
  for (int j = 0; j < len; j++) {
    b->x[start + j] = b->rb_x[j];
    b->y[start + j] = b->rb_y[j];
    b->z[start + j] = b->rb_z[j];
  }
}

/* SimCalcs::acceptMove, src/Metropolis/SimulationStep.cpp:794-803: accept a
 * decrease without drawing; otherwise accept when exp(-dE/kT) >= u. */
int orc_accept(double de, double kT, double u) {
  if (de < 0) return 1;
  return exp(-(de) / kT) >= u;
}

/* randomReal, src/Metropolis/Utilities/MathLibrary.cpp:31-33, with the
 * rand() value passed in (glibc RAND_MAX = 2147483647). */
double orc_random_real(double start, double end, int r) {
  return (end - start) * ((double)r / 2147483647) + start;
}

/* ---- Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11 "Parallel random
 * numbers: as easy as 1, 2, 3"), restated from the published description:
 * ten rounds of two 32x32->64 multiplies with the round keys bumped by the
 * Weyl constants between rounds. ---------------------------------------- */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                       uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Uniform in the open interval (0, 1) from 32 random bits. */
static double u01(uint32_t r) { return ((double)r + 0.5) * 2.3283064365386963e-10; }

/* Index in [0, n) from 32 random bits (multiply-shift, exact integer). */
static int uidx(uint32_t r, int n) { return (int)(((uint64_t)r * (uint64_t)n) >> 32); }

/* The trial move of step `step` of chain `chain` under key `seed`.  Counter
 * layout (step_lo, step_hi, chain, block): block 0 gives molecule, vertex,
 * dx, dy; block 1 gives dz and the three rotation draws; block 2 gives the
 * acceptance uniform.  Mode 0 draws Euler angles U(-maxR, maxR) degrees like
 * the reference; mode 1 draws a uniform axis on the sphere and an angle
 * U(-maxR, maxR) degrees. */
void orc_philox_move(uint64_t seed, uint32_t chain, uint64_t step, int n_mol,
                     const int* mol_len, double max_t, double max_r, int mode,
                     orc_move* mv) {
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t ctr[4] = {(uint32_t)step, (uint32_t)(step >> 32), chain, 0u};
  uint32_t a[4], c[4], d[4];
  orc_philox4x32_10(ctr, key, a);
  ctr[3] = 1u;
  orc_philox4x32_10(ctr, key, c);
  ctr[3] = 2u;
  orc_philox4x32_10(ctr, key, d);
  mv->mol = uidx(a[0], n_mol);
  mv->vertex = uidx(a[1], mol_len[mv->mol]);
  mv->mode = mode;
  mv->pad = 0;
  mv->dx = (2.0 * max_t) * u01(a[2]) - max_t;
  mv->dy = (2.0 * max_t) * u01(a[3]) - max_t;
  mv->dz = (2.0 * max_t) * u01(c[0]) - max_t;
  if (mode == 0) {
    mv->r0 = (2.0 * max_r) * u01(c[1]) - max_r;
    mv->r1 = (2.0 * max_r) * u01(c[2]) - max_r;
    mv->r2 = (2.0 * max_r) * u01(c[3]) - max_r;
    mv->r3 = 0.0;
  } else {
    double zc = 2.0 * u01(c[1]) - 1.0;
    double phi = 6.283185307179586 * u01(c[2]);
    double s = sqrt(1.0 - zc * zc);
    mv->r0 = s * cos(phi);
    mv->r1 = s * sin(phi);
    mv->r2 = zc;
    mv->r3 = (2.0 * max_r) * u01(c[3]) - max_r;
  }
  mv->u = u01(d[0]);
}

/* One Metropolis chain with Philox proposals: the loop body of
 * Simulation::run (src/Metropolis/Simulation.cpp:219-264) with NVT
 * acceptance.  Returns the running total energy (e0 + accepted dE). */
double orc_chain_run(orc_box* b, uint64_t seed, uint32_t chain, uint64_t step0,
                     int n_steps, int mode, double e0, orc_trace* trace,
                     long long* n_accepted) {
  double e = e0;
  long long acc = 0;
  orc_move mv;
  for (int s = 0; s < n_steps; s++) {
    orc_philox_move(seed, chain, step0 + (uint64_t)s, b->n_mol, b->mol_len,
                    b->max_translate, b->max_rotate, mode, &mv);
    double e_old = orc_mol_energy(b, mv.mol, 0);
    orc_apply_move(b, &mv);
    double e_new = orc_mol_energy(b, mv.mol, 0);
    double de = e_new - e_old;
    int ok = orc_accept(de, b->kT, mv.u);
    if (ok) {
      e += de;
      acc++;
    } else {
      orc_rollback(b, mv.mol);
    }
    if (trace) {
      trace[s].mol = mv.mol;
      trace[s].accepted = ok;
      trace[s].e_old = e_old;
      trace[s].e_new = e_new;
      trace[s].de = de;
      trace[s].u = mv.u;
    }
  }
  if (n_accepted) *n_accepted = acc;
  return e;
}

/* ---- multi-threaded driver for the CPU baseline ------------------------- */

typedef struct {
  orc_box* boxes;
  const uint64_t* seeds;
  int n_chains, n_steps, mode;
  uint64_t step0;
  int next;
  pthread_mutex_t lock;
  long long moves;
} mt_job;

static void* mt_worker(void* arg) {
  mt_job* j = (mt_job*)arg;
  long long local = 0;
  for (;;) {
    pthread_mutex_lock(&j->lock);
    int c = j->next++;
    pthread_mutex_unlock(&j->lock);
    if (c >= j->n_chains) break;
    orc_chain_run(&j->boxes[c], j->seeds[c], (uint32_t)c, j->step0, j->n_steps, j->mode,
                  0.0, NULL, NULL);
    local += j->n_steps;
  }
  pthread_mutex_lock(&j->lock);
  j->moves += local;
  pthread_mutex_unlock(&j->lock);
  return NULL;
}

/* Runs steps [step0, step0 + n_steps) of each chain (chain c is Philox
 * counter chain c), chains handed to n_threads worker threads in
 * index order (the reference has no threading; this is independent
 * single-chain runs side by side, as separate metrosim processes would be). */
double orc_chains_run_mt(orc_box* boxes, int n_chains, const uint64_t* seeds,
                         uint64_t step0, int n_steps, int mode, int n_threads,
                         long long* total_moves) {
  mt_job j;
  j.step0 = step0;
  j.boxes = boxes;
  j.seeds = seeds;
  j.n_chains = n_chains;
  j.n_steps = n_steps;
  j.mode = mode;
  j.next = 0;
  j.moves = 0;
  pthread_mutex_init(&j.lock, NULL);
  if (n_threads < 1) n_threads = 1;
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)n_threads);
  for (int t = 0; t < n_threads; t++) pthread_create(&th[t], NULL, mt_worker, &j);
  for (int t = 0; t < n_threads; t++) pthread_join(th[t], NULL);
  free(th);
  pthread_mutex_destroy(&j.lock);
  if (total_moves) *total_moves = j.moves;
  return 0.0;
}

/* ---- NPT volume move (restated; the reference's NPT path is not a valid
 * ensemble, see Ensemble.cpp:9-23 and SimulationStep.cpp:476-518) -------- */

/* Isotropic centre scaling about the origin by `scale`: every molecule is
 * shifted rigidly by (scale-1)*c, c its first primary atom, and the box
 * edges are multiplied by `scale`. */
void orc_resize_box_centres(orc_box* b, double scale) {
  double* c[3] = {b->x, b->y, b->z};
  for (int m = 0; m < b->n_mol; m++) {
    int p = b->pidx[b->mol_pidx_start[m]];
    int start = b->mol_start[m], end = start + b->mol_len[m];
    for (int d = 0; d < 3; d++) {
      double shift = (scale - 1.0) * c[d][p];
      for (int a = start; a < end; a++) c[d][a] += shift;
    }
  }
  for (int d = 0; d < 3; d++) b->size[d] *= scale;
}

/* Isobaric ln V move acceptance: accept when
 * u < exp(-(dU + P dV)/kT + (N+1) ln(V'/V)); P in kcal/mol/A^3. */
int orc_accept_volume(double de, double p_kcal_per_a3, double v_old, double v_new,
                      int n_mol, double kT, double u) {
  double arg = -(de + p_kcal_per_a3 * (v_new - v_old)) / kT +
               (double)(n_mol + 1) * log(v_new / v_old);
  if (arg >= 0) return 1;
  return exp(arg) >= u;
}

/* ---- device-resident chain form ----------------------------------------
 * Restated from the definition of the FP32 move (an independent CPU
 * implementation of the same arithmetic: every operation rounded once,
 * fused multiply-adds only where written as fmaf). */

static float u01f(uint32_t r) {
  return fmaf((float)(r >> 8), 5.9604644775390625e-08f, 2.98023223876953125e-08f);
}

/* sin/cos: Cody-Waite reduction by pi/2 in three parts, Taylor polynomials
 * of sin (to r^11) and cos (to r^12) by Horner's rule. */
void orc_sincos_f32(float x, float* sp, float* cp) {
  const float k = rintf(x * 0.636619772367581343f);
  float r = fmaf(-k, 1.5703125f, x);
  r = fmaf(-k, 4.83751296997070312e-04f, r);
  r = fmaf(-k, 7.54978995489188216e-08f, r);
  const float r2 = r * r;
  float s = fmaf(r2, -2.50521083854417188e-08f, 2.75573192239858907e-06f);
  s = fmaf(r2, s, -1.98412698412698413e-04f);
  s = fmaf(r2, s, 8.33333333333333333e-03f);
  s = fmaf(r2, s, -1.66666666666666667e-01f);
  s = fmaf(r2 * r, s, r);
  float c = fmaf(r2, 2.08767569878680990e-09f, -2.75573192239858907e-07f);
  c = fmaf(r2, c, 2.48015873015873016e-05f);
  c = fmaf(r2, c, -1.38888888888888889e-03f);
  c = fmaf(r2, c, 4.16666666666666667e-02f);
  c = fmaf(r2, c, -0.5f);
  c = fmaf(r2, c, 1.0f);
  const int q = ((int)k) & 3;
  *sp = (q == 0) ? s : (q == 1) ? c : (q == 2) ? -s : -c;
  *cp = (q == 0) ? c : (q == 1) ? -s : (q == 2) ? -c : s;
}

typedef struct { float w, x, y, z; } qf;

static qf q_mul(qf a, qf b) {
  qf r;
  r.w = ((a.w * b.w - a.x * b.x) - a.y * b.y) - a.z * b.z;
  r.x = ((a.w * b.x + a.x * b.w) + a.y * b.z) - a.z * b.y;
  r.y = ((a.w * b.y - a.x * b.z) + a.y * b.w) + a.z * b.x;
  r.z = ((a.w * b.z + a.x * b.y) - a.y * b.x) + a.z * b.w;
  return r;
}

static qf q_norm(qf a) {
  const float n = sqrtf(((a.w * a.w + a.x * a.x) + a.y * a.y) + a.z * a.z);
  qf r = {a.w / n, a.x / n, a.y / n, a.z / n};
  return r;
}

static void q_matrix(qf q, float* m) {
  const float xx = q.x * q.x, yy = q.y * q.y, zz = q.z * q.z;
  const float xy = q.x * q.y, xz = q.x * q.z, yz = q.y * q.z;
  const float wx = q.w * q.x, wy = q.w * q.y, wz = q.w * q.z;
  m[0] = 1.0f - 2.0f * (yy + zz);
  m[1] = 2.0f * (xy - wz);
  m[2] = 2.0f * (xz + wy);
  m[3] = 2.0f * (xy + wz);
  m[4] = 1.0f - 2.0f * (xx + zz);
  m[5] = 2.0f * (yz - wx);
  m[6] = 2.0f * (xz - wy);
  m[7] = 2.0f * (yz + wx);
  m[8] = 1.0f - 2.0f * (xx + yy);
}

static void m_vec(const float* m, const float* v, float* out) {
  out[0] = (m[0] * v[0] + m[1] * v[1]) + m[2] * v[2];
  out[1] = (m[3] * v[0] + m[4] * v[1]) + m[5] * v[2];
  out[2] = (m[6] * v[0] + m[7] * v[1]) + m[8] * v[2];
}

static qf q_axis(float kx, float ky, float kz, float a) {
  float s, c;
  orc_sincos_f32(0.5f * a, &s, &c);
  qf q = {c, s * kx, s * ky, s * kz};
  return q;
}

static int fix_step(float dx, float inv_s) { return (int)rintf(dx * inv_s); }

static double chain_coord(uint32_t A, float o, double L) {
  return (double)A * (L * 2.3283064365386963e-10) + (double)o;
}

static void chain_rows(orc_chain* c, int m) {
  orc_box* b = c->b;
  const int s = b->mol_start[m], n = b->mol_len[m];
  for (int a = s; a < s + n; a++) {
    b->x[a] = chain_coord(c->A[3 * m + 0], c->off[3 * a + 0], b->size[0]);
    b->y[a] = chain_coord(c->A[3 * m + 1], c->off[3 * a + 1], b->size[1]);
    b->z[a] = chain_coord(c->A[3 * m + 2], c->off[3 * a + 2], b->size[2]);
  }
}

void orc_fchain_init(orc_chain* c) {
  orc_box* b = c->b;
  for (int m = 0; m < b->n_mol; m++) {
    const int an = b->pidx[b->mol_pidx_start[m]];
    const double ax = b->x[an], ay = b->y[an], az = b->z[an];
    c->A[3 * m + 0] = (uint32_t)(uint64_t)llrint(ax * (4294967296.0 / b->size[0]));
    c->A[3 * m + 1] = (uint32_t)(uint64_t)llrint(ay * (4294967296.0 / b->size[1]));
    c->A[3 * m + 2] = (uint32_t)(uint64_t)llrint(az * (4294967296.0 / b->size[2]));
    c->q[4 * m + 0] = 1.0f;
    c->q[4 * m + 1] = c->q[4 * m + 2] = c->q[4 * m + 3] = 0.0f;
    const int s = b->mol_start[m], n = b->mol_len[m];
    for (int a = s; a < s + n; a++) {
      c->off[3 * a + 0] = c->tpl[3 * a + 0] = (float)(b->x[a] - ax);
      c->off[3 * a + 1] = c->tpl[3 * a + 1] = (float)(b->y[a] - ay);
      c->off[3 * a + 2] = c->tpl[3 * a + 2] = (float)(b->z[a] - az);
    }
    chain_rows(c, m);
  }
}

void orc_fchain_draw(const orc_chain* c, uint64_t seed, uint32_t chain, uint64_t step,
                    orc_movef* mv) {
  const orc_box* b = c->b;
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t ctr[4] = {(uint32_t)step, (uint32_t)(step >> 32), chain, 0u};
  uint32_t a[4], cc[4], d[4];
  orc_philox4x32_10(ctr, key, a);
  ctr[3] = 1u;
  orc_philox4x32_10(ctr, key, cc);
  ctr[3] = 2u;
  orc_philox4x32_10(ctr, key, d);
  mv->mol = uidx(a[0], b->n_mol);
  mv->vertex = uidx(a[1], b->mol_len[mv->mol]);
  const float max_t = (float)b->max_translate, max_r = (float)b->max_rotate;
  const float t2 = 2.0f * max_t;
  mv->dx = t2 * u01f(a[2]) - max_t;
  mv->dy = t2 * u01f(a[3]) - max_t;
  mv->dz = t2 * u01f(cc[0]) - max_t;
  const float r2 = 2.0f * max_r;
  const float deg = 0.0174532925199432958f;
  qf qd;
  if (c->rot_mode == 0) {
    const float ax = (r2 * u01f(cc[1]) - max_r) * deg;
    const float ay = (r2 * u01f(cc[2]) - max_r) * deg;
    const float az = (r2 * u01f(cc[3]) - max_r) * deg;
    const qf qx = q_axis(-1.0f, 0.0f, 0.0f, ax);
    const qf qy = q_axis(0.0f, -1.0f, 0.0f, ay);
    const qf qz = q_axis(0.0f, 0.0f, -1.0f, az);
    qd = q_mul(qz, q_mul(qy, qx));
  } else {
    const float zc = 2.0f * u01f(cc[1]) - 1.0f;
    const float phi = 6.28318530717958648f * u01f(cc[2]);
    const float sr = sqrtf(1.0f - zc * zc);
    float sp, cp;
    orc_sincos_f32(phi, &sp, &cp);
    const float ang = (r2 * u01f(cc[3]) - max_r) * deg;
    qd = q_axis(sr * cp, sr * sp, zc, ang);
  }
  mv->qw = qd.w; mv->qx = qd.x; mv->qy = qd.y; mv->qz = qd.z;
  mv->u = u01f(d[0]);
}

/* A move of chain molecule m proposed on the current state: its new
 * anchor, quaternion and offsets. */
typedef struct {
  int mol;
  uint32_t A[3];
  qf qn;
  float* off; /* [3 * mol_len] */
} fprop;

static void fchain_propose(const orc_chain* c, const orc_movef* mv, fprop* p) {
  const orc_box* b = c->b;
  const int m = mv->mol, a0 = b->mol_start[m], len = b->mol_len[m];
  qf q = {c->q[4 * m], c->q[4 * m + 1], c->q[4 * m + 2], c->q[4 * m + 3]};
  qf qd = {mv->qw, mv->qx, mv->qy, mv->qz};
  const qf qn = q_norm(q_mul(qd, q));
  float R[9];
  q_matrix(qn, R);
  const int v = a0 + mv->vertex;
  float onv[3];
  m_vec(R, &c->tpl[3 * v], onv);
  const float dl[3] = {(c->off[3 * v] - onv[0]) + mv->dx, (c->off[3 * v + 1] - onv[1]) + mv->dy,
                       (c->off[3 * v + 2] - onv[2]) + mv->dz};
  const float inv[3] = {(float)(4294967296.0 / b->size[0]), (float)(4294967296.0 / b->size[1]),
                        (float)(4294967296.0 / b->size[2])};
  p->mol = m;
  for (int k = 0; k < 3; k++) p->A[k] = c->A[3 * m + k] + (uint32_t)fix_step(dl[k], inv[k]);
  for (int i = 0; i < len; i++) m_vec(R, &c->tpl[3 * (a0 + i)], &p->off[3 * i]);
  p->qn = qn;
}

/* Molecule m of the state at anchor A and offsets off, its FP64 rows
 * refreshed. */
static void fchain_place(orc_chain* c, int m, const uint32_t* A, const float* off) {
  const orc_box* b = c->b;
  const int a0 = b->mol_start[m], len = b->mol_len[m];
  for (int k = 0; k < 3; k++) c->A[3 * m + k] = A[k];
  memcpy(&c->off[3 * a0], off, sizeof(float) * 3 * (size_t)len);
  chain_rows(c, m);
}

/* E_old and E_new of proposal p on the current state (the state is left
 * as it was); save holds 3 * mol_len floats. */
static void fchain_eval(orc_chain* c, const fprop* p, float* save, double* e_old, double* e_new) {
  orc_box* b = c->b;
  const int m = p->mol, a0 = b->mol_start[m], len = b->mol_len[m];
  uint32_t A0[3] = {c->A[3 * m], c->A[3 * m + 1], c->A[3 * m + 2]};
  memcpy(save, &c->off[3 * a0], sizeof(float) * 3 * (size_t)len);
  *e_old = orc_mol_energy(b, m, 0);
  fchain_place(c, m, p->A, p->off);
  *e_new = orc_mol_energy(b, m, 0);
  fchain_place(c, m, A0, save);
}

static int fchain_largest(const orc_box* b) {
  int big = 0;
  for (int m = 0; m < b->n_mol; m++)
    if (b->mol_len[m] > big) big = b->mol_len[m];
  return big;
}

/* The chain's Metropolis loop: draw, FP64 old energy, FP32 move of the
 * state, FP64 new energy, the reference's decision on the FP64 dE
 * (SimulationStep.cpp:794-803), commit or restore. */
double orc_fchain_run(orc_chain* c, uint64_t seed, uint32_t chain, uint64_t step0,
                     int n_steps, double e0, orc_trace* trace, long long* n_accepted) {
  orc_box* b = c->b;
  double e = e0;
  long long acc = 0;
  const int big = fchain_largest(b);
  float* save_off = (float*)malloc(sizeof(float) * 3 * (size_t)big);
  fprop p;
  p.off = (float*)malloc(sizeof(float) * 3 * (size_t)big);
  for (int st = 0; st < n_steps; st++) {
    orc_movef mv;
    orc_fchain_draw(c, seed, chain, step0 + (uint64_t)st, &mv);
    const int m = mv.mol;
    double e_old, e_new;
    fchain_propose(c, &mv, &p);
    fchain_eval(c, &p, save_off, &e_old, &e_new);
    const double de = e_new - e_old;
    const int ok = (de < 0) || (exp(-de / b->kT) >= (double)mv.u);
    if (ok) {
      e += de;
      acc++;
      fchain_place(c, m, p.A, p.off);
      c->q[4 * m] = p.qn.w; c->q[4 * m + 1] = p.qn.x; c->q[4 * m + 2] = p.qn.y;
      c->q[4 * m + 3] = p.qn.z;
    }
    if (trace) {
      trace[st].mol = m;
      trace[st].accepted = ok;
      trace[st].e_old = e_old;
      trace[st].e_new = e_new;
      trace[st].de = de;
      trace[st].u = (double)mv.u;
    }
  }
  free(p.off);
  free(save_off);
  if (n_accepted) *n_accepted = acc;
  return e;
}

/* Molecule m's primary positions (FP64, as its rows would hold them) at
 * anchor A and offsets off: out[3 * k + d] for primary k. */
static void fchain_prims(const orc_chain* c, int m, const uint32_t* A, const float* off,
                         double* out) {
  const orc_box* b = c->b;
  const int a0 = b->mol_start[m], ps = b->mol_pidx_start[m], pc = b->mol_pidx_count[m];
  for (int k = 0; k < pc; k++) {
    const int i = b->pidx[ps + k] - a0;
    for (int d = 0; d < 3; d++) out[3 * k + d] = chain_coord(A[d], off[3 * i + d], b->size[d]);
  }
}

/* The reference's in-range test (SimulationStep.cpp:317-342, the other
 * molecule's primary minus the moved one's) between primary sets pj (the
 * moved molecule, nj primaries) and pi (ni). */
static int prims_in_range(const orc_box* b, const double* pj, int nj, const double* pi, int ni) {
  for (int k1 = 0; k1 < nj; k1++)
    for (int k2 = 0; k2 < ni; k2++) {
      const double dx = orc_make_periodic(pi[3 * k2] - pj[3 * k1], b->size[0]);
      const double dy = orc_make_periodic(pi[3 * k2 + 1] - pj[3 * k1 + 1], b->size[1]);
      const double dz = orc_make_periodic(pi[3 * k2 + 2] - pj[3 * k1 + 2], b->size[2]);
      if (dx * dx + dy * dy + dz * dz <= b->cutoff * b->cutoff) return 1;
    }
  return 0;
}

/* The window form of the chain loop (the device's windowed kernel,
 * restated to check its rule exactly): windows of K steps; every step of a
 * window is proposed and evaluated on the state at the window's start; then,
 * in step order, a step's energies stand unless an earlier accepted step of
 * the window moved the same molecule (the move is then proposed again on the
 * current state) or moved a molecule that is in range of it (the reference's
 * test, either placement of either molecule); such a step is evaluated
 * again on the current state.  Otherwise orc_fchain_run: the same trace,
 * state and return value; *n_redo counts the steps evaluated again.
 * in_range_rule = 0 drops the in-range half of the rule (a planted mistake,
 * for the tests that show the rule is needed). */
double orc_fchain_run_window(orc_chain* c, uint64_t seed, uint32_t chain, uint64_t step0,
                             int n_steps, int K, double e0, orc_trace* trace,
                             long long* n_accepted, long long* n_redo, int in_range_rule) {
  orc_box* b = c->b;
  double e = e0;
  long long acc = 0, redo = 0;
  const int big = fchain_largest(b);
  int maxp = 0;
  for (int m = 0; m < b->n_mol; m++)
    if (b->mol_pidx_count[m] > maxp) maxp = b->mol_pidx_count[m];
  float* save = (float*)malloc(sizeof(float) * 3 * (size_t)big);
  fprop* p = (fprop*)malloc(sizeof(fprop) * (size_t)K);
  orc_movef* mv = (orc_movef*)malloc(sizeof(orc_movef) * (size_t)K);
  double* eo = (double*)malloc(sizeof(double) * (size_t)K);
  double* en = (double*)malloc(sizeof(double) * (size_t)K);
  int* ok = (int*)malloc(sizeof(int) * (size_t)K);
  /* primaries before and after each step: [K][2][3 * maxp] */
  double* pr = (double*)malloc(sizeof(double) * (size_t)K * 2 * 3 * (size_t)(maxp > 0 ? maxp : 1));
  for (int j = 0; j < K; j++) p[j].off = (float*)malloc(sizeof(float) * 3 * (size_t)big);
#define PR(j, t) (pr + ((size_t)(j) * 2 + (t)) * 3 * (size_t)maxp)
  for (int s0 = 0; s0 < n_steps; s0 += K) {
    const int nst = (n_steps - s0 < K) ? n_steps - s0 : K;
    for (int j = 0; j < nst; j++) {
      orc_fchain_draw(c, seed, chain, step0 + (uint64_t)(s0 + j), &mv[j]);
      fchain_propose(c, &mv[j], &p[j]);
      fchain_eval(c, &p[j], save, &eo[j], &en[j]);
    }
    for (int j = 0; j < nst; j++) {
      const int m = mv[j].mol, a0 = b->mol_start[m], nj = b->mol_pidx_count[m];
      int same = 0, near = 0;
      for (int i = 0; i < j; i++)
        if (ok[i] && mv[i].mol == m) same = 1;
      if (same) fchain_propose(c, &mv[j], &p[j]);
      fchain_prims(c, m, &c->A[3 * m], &c->off[3 * a0], PR(j, 0));
      fchain_prims(c, m, p[j].A, p[j].off, PR(j, 1));
      for (int i = 0; i < j && !same && !near && in_range_rule; i++) {
        if (!ok[i]) continue;
        const int ni = b->mol_pidx_count[mv[i].mol];
        for (int ti = 0; ti < 2 && !near; ti++)
          for (int tj = 0; tj < 2 && !near; tj++)
            near = prims_in_range(b, PR(j, tj), nj, PR(i, ti), ni);
      }
      if (same || near) {
        fchain_eval(c, &p[j], save, &eo[j], &en[j]);
        redo++;
      }
      const double de = en[j] - eo[j];
      ok[j] = (de < 0) || (exp(-de / b->kT) >= (double)mv[j].u);
      if (ok[j]) {
        e += de;
        acc++;
        fchain_place(c, m, p[j].A, p[j].off);
        c->q[4 * m] = p[j].qn.w; c->q[4 * m + 1] = p[j].qn.x; c->q[4 * m + 2] = p[j].qn.y;
        c->q[4 * m + 3] = p[j].qn.z;
      }
      if (trace) {
        orc_trace* t = &trace[s0 + j];
        t->mol = m;
        t->accepted = ok[j];
        t->e_old = eo[j];
        t->e_new = en[j];
        t->de = de;
        t->u = (double)mv[j].u;
      }
    }
  }
#undef PR
  for (int j = 0; j < K; j++) free(p[j].off);
  free(pr);
  free(ok);
  free(en);
  free(eo);
  free(mv);
  free(p);
  free(save);
  if (n_accepted) *n_accepted = acc;
  if (n_redo) *n_redo = redo;
  return e;
}

/* exp(x) for small |x| by its Taylor series to x^6, Horner's rule, each
 * operation rounded once (the device evaluates the same expression). */
static double exp_small(double x) {
  double p = 1.0 / 720.0;
  p = p * x + 1.0 / 120.0;
  p = p * x + 1.0 / 24.0;
  p = p * x + 1.0 / 6.0;
  p = p * x + 0.5;
  p = p * x + 1.0;
  p = p * x + 1.0;
  return p;
}

/* One isobaric ln V move of the chain state at step count `step`: draws
 * (Philox block 3: dlnv from word 0, u from word 1), every edge scaled by
 * exp(dlnv / 3) with the anchors' fixed-point fractions unchanged (centres
 * scale about the origin, geometry rigid), FP64 system energies at both
 * volumes (orc_system_energy on the state's rows), the isobaric criterion
 * exp(-(dU + P dV)/kT + (N + 1) dlnv) >= u, with dU including the change of
 * the long-range correction lrc_v / V (lrc_v = E_LRC * V; 0 for none).  Rejected outright (-1) when an
 * edge would fall to four times rad_max (the largest molecule radius).  *energy
 * becomes the FP64 energy of the kept volume (unchanged on -1).  Returns 1
 * accepted, 0 rejected. */
int orc_fchain_volume(orc_chain* c, uint64_t seed, uint32_t chain, uint64_t step,
                      double p_kcal, double max_dlnv, float rad_max, double lrc_v, double* energy,
                      double* e_old, double* e_new, double* dlnv_out, double* u_out) {
  orc_box* b = c->b;
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t ctr[4] = {(uint32_t)step, (uint32_t)(step >> 32), chain, 3u};
  uint32_t r[4];
  orc_philox4x32_10(ctr, key, r);
  const double dlnv = (2.0 * max_dlnv) * u01(r[0]) + (-max_dlnv);
  const double u = u01(r[1]);
  if (dlnv_out) *dlnv_out = dlnv;
  if (u_out) *u_out = u;
  const double s = exp_small(dlnv / 3.0);
  double Ln[3], Lo[3], Lmin = 1e300;
  for (int k = 0; k < 3; k++) {
    Lo[k] = b->size[k];
    Ln[k] = Lo[k] * s;
    if (Ln[k] < Lmin) Lmin = Ln[k];
  }
  if ((double)rad_max >= 0.25 * Lmin) return -1;
  const double eo = orc_system_energy(b);
  for (int k = 0; k < 3; k++) b->size[k] = Ln[k];
  for (int m = 0; m < b->n_mol; m++) chain_rows(c, m);
  const double en = orc_system_energy(b);
  if (e_old) *e_old = eo;
  if (e_new) *e_new = en;
  const double vo = Lo[0] * Lo[1] * Lo[2];
  const double vn = Ln[0] * Ln[1] * Ln[2];
  const double d_lrc = lrc_v / vn - lrc_v / vo;
  const double arg =
      -((en - eo) + d_lrc + p_kcal * (vn - vo)) / b->kT + (double)(b->n_mol + 1) * dlnv;
  const int ok = (arg >= 0.0) || (exp(arg) >= u);
  if (ok) {
    *energy = en;
  } else {
    for (int k = 0; k < 3; k++) b->size[k] = Lo[k];
    for (int m = 0; m < b->n_mol; m++) chain_rows(c, m);
    *energy = eo;
  }
  return ok;
}

/* ---- synthetic initial configuration (input generation, not the path) ---
 *
 * Centres by random sequential addition: points uniform in [0, L)^3, each
 * candidate closer than dmin (minimum image) to a placed one redrawn, drawn
 * from xoshiro256** seeded by splitmix64 (Blackman & Vigna 2018, restated
 * from their published description).  It places the same points as the
 * product's input builder for the same arguments, so the CPU baseline can
 * build its workload without loading the product library.  Returns 0, 1
 * (bad argument) or 2 (no room). */
static uint64_t orc_splitmix64(uint64_t* s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static uint64_t orc_rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static double orc_xoshiro_u01(uint64_t st[4]) {
  const uint64_t r = orc_rotl64(st[1] * 5, 7) * 9;
  const uint64_t t = st[1] << 17;
  st[2] ^= st[0];
  st[3] ^= st[1];
  st[1] ^= st[2];
  st[0] ^= st[3];
  st[2] ^= t;
  st[3] = orc_rotl64(st[3], 45);
  return (double)(r >> 11) * 0x1.0p-53;
}

int orc_build_centres(int n, double L, double dmin, uint64_t seed, double* out) {
  if (n < 0 || !(L > 0) || !(dmin >= 0) || (n > 0 && !out)) return 1;
  if (n == 0) return 0;
  int nc = dmin > 0 ? (int)floor(L / dmin) : 1;
  if (nc < 3) nc = 1;
  if (nc > 512) nc = 512;
  const double cw = L / nc;
  const size_t ncell = (size_t)nc * nc * nc;
  /* per-cell singly linked lists of placed points (head per cell, next per point) */
  int* head = (int*)malloc(sizeof(int) * ncell);
  int* next = (int*)malloc(sizeof(int) * (size_t)n);
  if (!head || !next) {
    free(head);
    free(next);
    return 2;
  }
  for (size_t i = 0; i < ncell; i++) head[i] = -1;
  uint64_t st[4], sd = seed;
  for (int i = 0; i < 4; i++) st[i] = orc_splitmix64(&sd);
  const double d2 = dmin * dmin;
  const long long max_tries = 2000LL * n + 100000;
  long long tries = 0;
  int k = 0, rc = 0;
  while (k < n) {
    if (++tries > max_tries) {
      rc = 2;
      break;
    }
    double p[3];
    for (int d = 0; d < 3; d++) p[d] = orc_xoshiro_u01(st) * L;
    int c[3];
    for (int d = 0; d < 3; d++) {
      c[d] = (int)(p[d] / cw);
      if (c[d] >= nc) c[d] = nc - 1;
      if (nc < 3) c[d] = 0;
    }
    int ok = 1;
    const int span = nc >= 3 ? 1 : 0;
    for (int a = -span; a <= span && ok; a++)
      for (int b = -span; b <= span && ok; b++)
        for (int e = -span; e <= span && ok; e++) {
          const int ca = (c[0] + a + nc) % nc, cb = (c[1] + b + nc) % nc, ce = (c[2] + e + nc) % nc;
          for (int j = head[((size_t)ca * nc + cb) * nc + ce]; j >= 0 && ok; j = next[j]) {
            double r2 = 0;
            for (int d = 0; d < 3; d++) {
              double dx = out[3 * j + d] - p[d];
              dx -= L * nearbyint(dx / L);
              r2 += dx * dx;
            }
            if (r2 < d2) ok = 0;
          }
        }
    if (!ok) continue;
    const size_t cell = ((size_t)c[0] * nc + c[1]) * nc + c[2];
    next[k] = head[cell];
    head[cell] = k;
    for (int d = 0; d < 3; d++) out[3 * k + d] = p[d];
    k++;
  }
  free(head);
  free(next);
  return rc;
}

/* ---- flexible molecules ------------------------------------------------------
 *
 * The reference compiles these functions but calls them only with
 * ENABLE_INTRA true (src/Metropolis/SimulationStep.h:15 sets it false); the
 * restatement follows them as they run with it true: molecule energies carry
 * the intramolecular term (SimulationStep.cpp:15-18), a trial move is the
 * rigid move followed by the intramolecular one (:424-428) and a rollback
 * also restores the bond lengths and angle sizes (:731-749).  Random draws
 * come from the C library's rand(), as the reference's randomReal
 * (MathLibrary.cpp:31-33) takes them. */

static double intra_random_real(double start, double end) {
  return orc_random_real(start, end, rand());
}

/* SimCalcs::bondEnergy, src/Metropolis/SimulationStep.cpp:241-255:
 * sum of k (eq - length)^2 over the molecule's variable bonds. */
double orc_bond_energy(const orc_topo* t, int mol) {
  double out = 0;
  int s = t->mol_bond_start[mol], e = s + t->mol_bond_count[mol];
  for (int i = s; i < e; i++) {
    if (t->bond_var[i]) {
      double diff = t->bond_eq[i] - t->bond_len[i];
      out += t->bond_k[i] * diff * diff;
    }
  }
  return out;
}

/* SimCalcs::angleEnergy, :131-146 (sizes in degrees, as tracked). */
double orc_angle_energy(const orc_topo* t, int mol) {
  double out = 0;
  int s = t->mol_angle_start[mol], e = s + t->mol_angle_count[mol];
  for (int i = s; i < e; i++) {
    if (t->angle_var[i]) {
      double diff = t->angle_eq[i] - t->angle_size[i];
      out += t->angle_k[i] * diff * diff;
    }
  }
  return out;
}

/* SimCalcs::calcIntraMolecularEnergy, :80-129: angle and bond terms when the
 * box has variable angles / bonds, then, when it has either, the LJ and
 * Coulomb terms of every atom pair i < j of the molecule not excluded,
 * halved for the fudge pairs; no cutoff, minimum image per pair, and the
 * SimCalcs pair functions (blending by sqrt|a b|, so sites with negative
 * sigma or epsilon take part here). */
double orc_intra_energy(const orc_box* b, const orc_topo* t, int mol) {
  double out = 0.0;
  if (t->flex_angles) out += orc_angle_energy(t, mol);
  if (t->flex_bonds) out += orc_bond_energy(t, mol);
  if (t->flex_bonds || t->flex_angles) {
    const int s = b->mol_start[mol], e = s + b->mol_len[mol];
    const int ty = t->mol_type[mol], n = t->type_natom[ty];
    const unsigned char* code = t->pair_code + t->type_off[ty];
    for (int i = s; i < e; i++) {
      for (int j = i + 1; j < e; j++) {
        const int li = i - s, lj = j - s;
        /* an atom beyond the type's first molecule's length finds no list
         * entry: full weight */
        const int c = (li < n && lj < n) ? code[li * n + lj] : 2;
        const double fudge = c == 0 ? 0.0 : (c == 1 ? 0.5 : 1.0);
        if (fudge > 0.0) {
          double r2 = orc_atom_dist2(b, i, j);
          double r = sqrt(r2);
          double energy = orc_lj(b, i, j, r2);
          energy += orc_charge(b, i, j, r);
          out += fudge * energy;
        }
      }
    }
  }
  return out;
}

/* SimCalcs::find / unionAtoms, :777-792 (local atom indexes). */
static int uf_find(int* p, int a) {
  int r = a;
  while (p[r] != r) r = p[r];
  while (p[a] != r) {
    int nx = p[a];
    p[a] = r;
    a = nx;
  }
  return r;
}
static void uf_union(int* p, int a, int c) {
  int ra = uf_find(p, a), rc = uf_find(p, c);
  if (ra != rc) p[ra] = rc;
}

/* SimCalcs::stretchBond, :257-315: the molecule's atoms split into the two
 * sides of bond `bond` (the union of every other bond of the molecule); the
 * side of its second atom moves by +dist/2 along the bond's unit vector and
 * every other atom by -dist/2; the tracked length grows by dist.  A bond in a
 * ring (one side) is left alone. */
void orc_stretch_bond(orc_box* b, orc_topo* t, int mol, int bond, double dist) {
  const int bs = t->mol_bond_start[mol], be = bs + t->mol_bond_count[mol];
  const int start = b->mol_start[mol], len = b->mol_len[mol];
  const int e1 = t->bond_a1[bs + bond], e2 = t->bond_a2[bs + bond];
  int* p = t->uf;
  for (int i = 0; i < len; i++) p[i] = i;
  for (int i = bs; i < be; i++) {
    if (i == bond + bs) continue;
    uf_union(p, t->bond_a1[i] - start, t->bond_a2[i] - start);
  }
  const int side1 = uf_find(p, e1 - start), side2 = uf_find(p, e2 - start);
  if (side1 == side2) return;
  double v[3], denon = 0.0;
  v[0] = b->x[e2] - b->x[e1];
  v[1] = b->y[e2] - b->y[e1];
  v[2] = b->z[e2] - b->z[e1];
  for (int k = 0; k < 3; k++) denon += v[k] * v[k];
  denon = sqrt(denon);
  for (int k = 0; k < 3; k++) v[k] = v[k] / denon / 2.0;
  double* c[3] = {b->x, b->y, b->z};
  for (int i = 0; i < len; i++) {
    if (uf_find(p, i) == side2) {
      for (int k = 0; k < 3; k++) c[k][i + start] += v[k] * dist;
    } else {
      for (int k = 0; k < 3; k++) c[k][i + start] -= v[k] * dist;
    }
  }
  t->bond_len[bs + bond] += dist;
}

/* SimCalcs::expandAngle, :148-239: with the bonds touching the middle atom
 * removed, the component of the first end turns by -deg and that of the
 * second end by +deg about the unit normal of the plane (mid - end1,
 * mid - end2) through the middle atom (Rodrigues' rotation); the tracked size
 * grows by deg.  Both ends in one component (a ring) leave the angle alone.
 * DEG2RAD is the reference's constant, whose digits differ from pi's after
 * the seventh. */
void orc_expand_angle(orc_box* b, orc_topo* t, int mol, int angle, double deg) {
  const int bs = t->mol_bond_start[mol], be = bs + t->mol_bond_count[mol];
  const int as = t->mol_angle_start[mol];
  const int start = b->mol_start[mol], len = b->mol_len[mol];
  const int end1 = t->angle_a1[as + angle], end2 = t->angle_a2[as + angle];
  const int mid = t->angle_mid[as + angle];
  int* p = t->uf;
  for (int i = 0; i < len; i++) p[i] = i;
  for (int i = bs; i < be; i++) {
    int a1 = t->bond_a1[i], a2 = t->bond_a2[i];
    if (a1 == mid || a2 == mid) continue;
    uf_union(p, a1 - start, a2 - start);
  }
  const int group1 = uf_find(p, end1 - start), group2 = uf_find(p, end2 - start);
  if (group1 == group2) return;
  const double DEG2RAD = 3.14159256358979323846264 / 180.0;
  double* c[3] = {b->x, b->y, b->z};
  double e1m[3], e2m[3], normal[3], mv[3];
  for (int k = 0; k < 3; k++) {
    e1m[k] = c[k][mid] - c[k][end1];
    e2m[k] = c[k][mid] - c[k][end2];
    mv[k] = c[k][mid];
  }
  normal[0] = e1m[1] * e2m[2] - e2m[1] * e1m[2];
  normal[1] = e2m[0] * e1m[2] - e1m[0] * e2m[2];
  normal[2] = e1m[0] * e2m[1] - e2m[0] * e1m[1];
  double nl = 0.0;
  for (int k = 0; k < 3; k++) nl += normal[k] * normal[k];
  nl = sqrt(nl);
  for (int k = 0; k < 3; k++) normal[k] = normal[k] / nl;
  for (int i = start; i < start + len; i++) {
    double theta;
    const int g = uf_find(p, i - start);
    if (g == group1)
      theta = deg * -DEG2RAD;
    else if (g == group2)
      theta = deg * DEG2RAD;
    else
      continue;
    double pt[3], cr[3], dot = 0.0;
    for (int k = 0; k < 3; k++) {
      pt[k] = c[k][i] - mv[k];
      dot += pt[k] * normal[k];
    }
    cr[0] = normal[1] * pt[2] - pt[1] * normal[2];
    cr[1] = pt[0] * normal[2] - normal[0] * pt[2];
    cr[2] = normal[0] * pt[1] - pt[0] * normal[1];
    for (int k = 0; k < 3; k++) {
      pt[k] = (normal[k] * dot * (1 - cos(theta)) + pt[k] * cos(theta) + cr[k] * sin(theta));
      c[k][i] = pt[k] + mv[k];
    }
  }
  t->angle_size[as + angle] += deg;
}

/* SimCalcs::saveBonds / saveAngles, :678-701. */
void orc_save_intra(orc_topo* t, int mol) {
  int s = t->mol_bond_start[mol], n = t->mol_bond_count[mol];
  for (int i = 0; i < n; i++) t->bond_len_rb[i + s] = t->bond_len[i + s];
  s = t->mol_angle_start[mol];
  n = t->mol_angle_count[mol];
  for (int i = 0; i < n; i++) t->angle_size_rb[i + s] = t->angle_size[i + s];
}

/* SimCalcs::rollbackAngles / rollbackBonds, :751-775. */
void orc_rollback_intra(orc_topo* t, int mol) {
  int s = t->mol_angle_start[mol], n = t->mol_angle_count[mol];
  for (int i = s; i < s + n; i++) t->angle_size[i] = t->angle_size_rb[i];
  s = t->mol_bond_start[mol];
  n = t->mol_bond_count[mol];
  for (int i = s; i < s + n; i++) t->bond_len[i] = t->bond_len_rb[i];
}

/* Draws the distinct indexes of the bonds or angles to move, as the
 * reference inserts (int)randomReal(0, count) into a std::set until it holds
 * `want` of them (:599-601, :631-633), and returns them in ascending order
 * (the set's iteration order).  A draw equal to count (rand() == RAND_MAX) is
 * kept as count - 1 here; the reference would index past the molecule. */
static int draw_set(int want, int count, int* out) {
  int n = 0;
  while (n < want) {
    int v = (int)intra_random_real(0, count);
    if (v >= count) v = count - 1;
    int pos = 0;
    while (pos < n && out[pos] < v) pos++;
    if (pos < n && out[pos] == v) continue;
    for (int k = n; k > pos; k--) out[k] = out[k - 1];
    out[pos] = v;
    n++;
  }
  return n;
}

/* SimCalcs::intramolecularMove, :568-675 (ENABLE_BOND 1, ENABLE_ANGLE 1,
 * ENABLE_DIHEDRAL 0, ENABLE_TUNING true, TARGET_RATIO 0.4, RATIO_MARGIN
 * 1e-4 from SimulationStep.h:16-22): save the rows; stretch a random subset
 * of the bonds, an MC test on the intramolecular energy that only counts
 * acceptances (it never rolls back), the same for the angles, and every 1000
 * steps the widths scaled toward a 40 % acceptance.  The angle width test
 * reads the width itself where the bond test reads the ratio's distance
 * (:666), as the reference does. */
void orc_intramolecular_move(orc_box* b, orc_topo* t, int mol) {
  orc_save_intra(t, mol);
  const int n_types = 2;  /* ENABLE_BOND + ENABLE_ANGLE + ENABLE_DIHEDRAL */
  const double intra_scale = 0.25 + (0.75 / (double)n_types);
  double scale;
  int idx[64];
  double new_e = 0, cur_e = orc_intra_energy(b, t, mol);
  const int n_bonds = t->mol_bond_count[mol], bond_start = t->mol_bond_start[mol];
  const int n_angles = t->mol_angle_count[mol], angle_start = t->mol_angle_start[mol];
  const double bond_delta = t->max_bond_delta, angle_delta = t->max_angle_delta;
  if (t->flex_bonds) {
    int n = n_bonds;
    if (n > 3) {
      n = (int)intra_random_real(2, n_bonds);
      if (n > t->max_intra_moves) n = t->max_intra_moves;
    }
    scale = 0.25 + (0.75 / (double)n) * intra_scale;
    t->bond_moves += n;
    draw_set(n, n_bonds, idx);
    for (int k = 0; k < n; k++) {
      double d = scale * intra_random_real(-bond_delta, bond_delta);
      if (t->bond_var[bond_start + idx[k]]) orc_stretch_bond(b, t, mol, idx[k], d);
    }
    new_e = orc_intra_energy(b, t, mol);
    if (orc_accept(new_e - cur_e, b->kT, new_e - cur_e < 0 ? 0.0
                                                           : intra_random_real(0.0, 1.0)))
      t->bond_accepted += n;
    cur_e = new_e;
  }
  if (t->flex_angles) {
    int n = n_angles;
    if (n > 3) {
      n = (int)intra_random_real(2, n_angles);
      if (n > t->max_intra_moves) n = t->max_intra_moves;
    }
    scale = 0.25 + (0.75 / (double)n) * intra_scale;
    t->angle_moves += n;
    draw_set(n, n_angles, idx);
    for (int k = 0; k < n; k++) {
      double d = scale * intra_random_real(-angle_delta, angle_delta);
      if (t->angle_var[angle_start + idx[k]]) orc_expand_angle(b, t, mol, idx[k], d);
    }
    new_e = orc_intra_energy(b, t, mol);
    if (orc_accept(new_e - cur_e, b->kT, new_e - cur_e < 0 ? 0.0
                                                           : intra_random_real(0.0, 1.0)))
      t->angle_accepted += n;
    cur_e = new_e;
  }
  if (t->step_num != 0 && (t->step_num % 1000) == 0) {
    double bond_ratio = (double)t->bond_accepted / t->bond_moves;
    double angle_ratio = (double)t->angle_accepted / t->angle_moves;
    double diff = bond_ratio - 0.4;
    if (fabs(diff) > 0.0001) t->max_bond_delta += t->max_bond_delta * diff;
    diff = angle_ratio - 0.4;
    if (fabs(angle_delta) > 0.0001) t->max_angle_delta += t->max_angle_delta * diff;
    t->bond_accepted = t->bond_moves = 0;
    t->angle_accepted = t->angle_moves = 0;
  }
}

/* SimulationStep::calcSystemEnergy with the intramolecular term (:40-71). */
double orc_system_energy_intra(const orc_box* b, const orc_topo* t) {
  double total = 0;
  for (int m = 0; m < b->n_mol; m++)
    total += orc_mol_energy(b, m, m) + orc_intra_energy(b, t, m);
  return total;
}

/* Simulation::run's NVT loop (Simulation.cpp:219-264) with the
 * intramolecular term and move: choose (rand), E_old, the seven draws of
 * intermolecularMove and the move, the intramolecular move, E_new, accept or
 * roll back everything, then the step counter. */
double orc_run_plain_intra(orc_box* b, orc_topo* t, int steps, double e0, int* accepted) {
  double e = e0;
  int acc = 0;
  for (int s = 0; s < steps; s++) {
    int mol = (int)intra_random_real(0, b->n_mol);
    if (mol >= b->n_mol) mol = b->n_mol - 1;
    double old_e = orc_mol_energy(b, mol, 0) + orc_intra_energy(b, t, mol);
    orc_move mv;
    memset(&mv, 0, sizeof(mv));
    mv.mol = mol;
    const int len = b->mol_len[mol];
    mv.vertex = (int)intra_random_real(0, len);
    if (mv.vertex >= len) mv.vertex = len - 1;
    mv.dx = intra_random_real(-b->max_translate, b->max_translate);
    mv.dy = intra_random_real(-b->max_translate, b->max_translate);
    mv.dz = intra_random_real(-b->max_translate, b->max_translate);
    mv.r0 = intra_random_real(-b->max_rotate, b->max_rotate);
    mv.r1 = intra_random_real(-b->max_rotate, b->max_rotate);
    mv.r2 = intra_random_real(-b->max_rotate, b->max_rotate);
    orc_apply_move(b, &mv);
    orc_intramolecular_move(b, t, mol);
    double new_e = orc_mol_energy(b, mol, 0) + orc_intra_energy(b, t, mol);
    const double de = new_e - old_e;
    if (orc_accept(de, b->kT, de < 0 ? 0.0 : intra_random_real(0.0, 1.0))) {
      acc++;
      e += de;
    } else {
      orc_rollback(b, mol);
      orc_rollback_intra(t, mol);
    }
    t->step_num++;
  }
  if (accepted) *accepted = acc;
  return e;
}
