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
