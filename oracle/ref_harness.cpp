// ref_harness.cpp -- white-box harness around the REFERENCE's own compiled
// CPU path (MCGPU built from its unmodified sources by oracle/Makefile into
// oracle/_ref/).  TEST INFRASTRUCTURE ONLY: it pins the oracle restatement
// (mcgpu_oracle.c) and generates the golden vectors under tests/golden/.
//
// It builds a SimBox directly from structure-of-arrays inputs (the layout of
// src/Metropolis/SimBox.h:120-149, filled as SimBoxBuilder.cpp:44-135 and
// :282-299 fill it), points GPUCopy at the host rows (GPUCopy.cpp:97-110 with
// parallel=false) and then calls the reference's own functions.
#include <cstdlib>
#include <cstring>

#include "Metropolis/Box.h"
#include "Metropolis/BruteForceStep.h"
#include "Metropolis/GPUCopy.h"
#include "Metropolis/SerialSim/SerialCalcs.h"
#include "Metropolis/SimBox.h"
#include "Metropolis/SimBoxBuilder.h"
#include "Metropolis/SimulationArgs.h"
#include "Metropolis/SimulationStep.h"
#include "Metropolis/Utilities/FileUtilities.h"
#include "Metropolis/Utilities/MathLibrary.h"

namespace {
SimBox* g_sb = nullptr;
BruteForceStep* g_step = nullptr;
// ref_load: the reference's Box and the SimBox built from it
Box* g_lbox = nullptr;
SimBox* g_lsb = nullptr;
long g_lstart = 0, g_lsteps = 0;

template <class T>
T* copy_row(const T* src, int n) {
  T* d = new T[n > 0 ? n : 1];
  if (n > 0) std::memcpy(d, src, sizeof(T) * n);
  return d;
}
}  // namespace

extern "C" {

// Builds the global SimBox.  Rows not used by the rigid-molecule path
// (bonds, angles, NLC) are allocated empty, as SimBoxBuilder leaves them for
// a molecule type with no flexible bonds or angles.
int ref_box_create(int n_mol, int n_atom, int n_pidx, const double* x,
                   const double* y, const double* z, const double* sigma,
                   const double* epsilon, const double* charge,
                   const int* mol_start, const int* mol_len,
                   const int* mol_pidx_start, const int* mol_pidx_count,
                   const int* pidx, const double* size, double cutoff,
                   double temperature, double max_t, double max_r) {
  SimBox* sb = new SimBox();
  sb->stepNum = 0;
  sb->size = copy_row(size, 3);
  sb->temperature = temperature;
  sb->kT = temperature * kBoltz;  // SimBoxBuilder.cpp:29
  sb->cutoff = cutoff;
  sb->maxTranslate = max_t;
  sb->maxRotate = max_r;
  sb->maxBondDelta = 0;
  sb->maxAngleDelta = 0;
  sb->numSteps = 0;
  sb->maxIntraMoves = 15;
  sb->numMolecules = n_mol;
  sb->numAtoms = n_atom;
  sb->numPIdxes = n_pidx;
  sb->numBonds = sb->numAngles = sb->numDihedrals = 0;
  int largest = 0;
  for (int i = 0; i < n_mol; i++)
    if (mol_len[i] > largest) largest = mol_len[i];
  sb->largestMol = largest;

  sb->moleculeData = new int*[MOL_DATA_SIZE];
  for (int r = 0; r < MOL_DATA_SIZE; r++) {
    sb->moleculeData[r] = new int[n_mol];
    std::memset(sb->moleculeData[r], 0, sizeof(int) * n_mol);
  }
  std::memcpy(sb->moleculeData[MOL_START], mol_start, sizeof(int) * n_mol);
  std::memcpy(sb->moleculeData[MOL_LEN], mol_len, sizeof(int) * n_mol);
  std::memcpy(sb->moleculeData[MOL_PIDX_START], mol_pidx_start, sizeof(int) * n_mol);
  std::memcpy(sb->moleculeData[MOL_PIDX_COUNT], mol_pidx_count, sizeof(int) * n_mol);
  sb->primaryIndexes = copy_row(pidx, n_pidx);

  sb->atomCoordinates = new Real*[NUM_DIMENSIONS];
  sb->atomCoordinates[X_COORD] = copy_row(x, n_atom);
  sb->atomCoordinates[Y_COORD] = copy_row(y, n_atom);
  sb->atomCoordinates[Z_COORD] = copy_row(z, n_atom);
  sb->rollBackCoordinates = new Real*[NUM_DIMENSIONS];
  for (int d = 0; d < NUM_DIMENSIONS; d++) {
    sb->rollBackCoordinates[d] = new Real[largest];
    std::memset(sb->rollBackCoordinates[d], 0, sizeof(Real) * largest);
  }
  sb->atomData = new Real*[ATOM_DATA_SIZE];
  sb->atomData[ATOM_SIGMA] = copy_row(sigma, n_atom);
  sb->atomData[ATOM_EPSILON] = copy_row(epsilon, n_atom);
  sb->atomData[ATOM_CHARGE] = copy_row(charge, n_atom);

  sb->bondLengths = new Real[1];
  sb->rollBackBondLengths = new Real[1];
  sb->bondData = new Real*[BOND_DATA_SIZE];
  for (int r = 0; r < BOND_DATA_SIZE; r++) sb->bondData[r] = new Real[1];
  sb->angleSizes = new Real[1];
  sb->rollBackAngleSizes = new Real[1];
  sb->angleData = new Real*[ANGLE_DATA_SIZE];
  for (int r = 0; r < ANGLE_DATA_SIZE; r++) sb->angleData[r] = new Real[1];
  sb->numBondMoves = sb->numAcceptedBondMoves = 0;
  sb->numAngleMoves = sb->numAcceptedAngleMoves = 0;
  sb->hasFlexibleBonds = false;
  sb->hasFlexibleAngles = false;
  sb->useNLC = false;
  sb->unionFindParent = new int[largest];
  sb->excludeAtoms = nullptr;
  sb->fudgeAtoms = nullptr;

  g_sb = sb;
  GPUCopy::setParallel(false);
  GPUCopy::copyIn(sb);
  delete g_step;
  g_step = new BruteForceStep(sb);  // sets SimCalcs::sb (SimulationStep.cpp:11-13)
  return 0;
}

// BruteForceCalcs::calcMolecularEnergyContribution (BruteForceStep.cpp:15-46).
double ref_mol_energy(int curr, int start) {
  return g_step->calcMolecularEnergyContribution(curr, start);
}

// SimulationStep::calcSystemEnergy (SimulationStep.cpp:40-71); prints the
// reference's VERBOSE breakdown to stdout.
double ref_system_energy(void) {
  Real lj = 0, charge = 0;
  return g_step->calcSystemEnergy(lj, charge, g_sb->numMolecules);
}

// The body of SimCalcs::intermolecularMove (SimulationStep.cpp:520-566) with
// the seven draws supplied by the caller; every coordinate update goes
// through the reference's own rotateAtom / translateAtom / keepMoleculeInBox.
void ref_apply_move(int mol, int vertex, double dx, double dy, double dz,
                    double rx, double ry, double rz) {
  int start = g_sb->moleculeData[MOL_START][mol];
  int len = g_sb->moleculeData[MOL_LEN][mol];
  Real** rb = GPUCopy::rollBackCoordinatesPtr();
  Real** ac = GPUCopy::atomCoordinatesPtr();
  for (int i = 0; i < len; i++) {
    for (int d = 0; d < NUM_DIMENSIONS; d++) rb[d][i] = ac[d][start + i];
    if (i == vertex) continue;
    SimCalcs::rotateAtom(start + i, start + vertex, rx, ry, rz, ac);
    SimCalcs::translateAtom(start + i, dx, dy, dz, ac);
  }
  ac[0][start + vertex] += dx;
  ac[1][start + vertex] += dy;
  ac[2][start + vertex] += dz;
  SimCalcs::keepMoleculeInBox(mol, ac, GPUCopy::moleculeDataPtr(),
                              GPUCopy::primaryIndexesPtr(), GPUCopy::sizePtr());
}

// The reference's own SimCalcs::intermolecularMove, drawing from rand().
void ref_intermolecular_move(int mol) { SimCalcs::intermolecularMove(mol); }

// SimCalcs::rollback (SimulationStep.cpp:731-749).
void ref_rollback(int mol) { SimCalcs::rollback(mol); }

// SimCalcs::acceptMove (SimulationStep.cpp:794-803), draws rand() when dE>=0.
int ref_accept(double de) { return SimCalcs::acceptMove(de) ? 1 : 0; }

// SimulationStep::chooseMolecule (SimulationStep.cpp:25-27).
int ref_choose_molecule(void) { return g_step->chooseMolecule(g_sb); }

void ref_seed(int s) { seed(s); }
int ref_rand(void) { return rand(); }

// Wraps every molecule by its primary atom as Simulation::run does before
// the loop (Simulation.cpp:70-72), via the SimBox copy of keepMoleculeInBox.
void ref_wrap_all(void) {
  for (int m = 0; m < g_sb->numMolecules; m++)
    SimCalcs::keepMoleculeInBox(m, GPUCopy::atomCoordinatesPtr(),
                                GPUCopy::moleculeDataPtr(),
                                GPUCopy::primaryIndexesPtr(), GPUCopy::sizePtr());
}

void ref_get_coords(double* x, double* y, double* z) {
  std::memcpy(x, g_sb->atomCoordinates[X_COORD], sizeof(double) * g_sb->numAtoms);
  std::memcpy(y, g_sb->atomCoordinates[Y_COORD], sizeof(double) * g_sb->numAtoms);
  std::memcpy(z, g_sb->atomCoordinates[Z_COORD], sizeof(double) * g_sb->numAtoms);
}

// The main loop of Simulation::run (Simulation.cpp:219-264) for the NVT
// brute-force strategy, calling the reference's own step object, ensemble
// rule and RNG; returns the running energy started at e0.
double ref_run_plain(int steps, double e0, int* accepted) {
  double e = e0;
  int acc = 0;
  for (int move = 0; move < steps; move++) {
    int idx = g_step->chooseMolecule(g_sb);
    double old_e = g_step->calcMoleculeEnergy(idx, 0);
    g_step->changeMolecule(idx, g_sb);
    double new_e = g_step->calcMoleculeEnergy(idx, 0);
    if (SimCalcs::acceptMove(new_e - old_e)) {
      acc++;
      e += new_e - old_e;
    } else {
      g_step->rollback(idx, g_sb);
    }
    g_sb->stepNum++;
  }
  if (accepted) *accepted = acc;
  return e;
}

// ---- the reference's own file pipeline ---------------------------------------
//
// Loads a .config (z-matrix + OPLS table on the FCC lattice) or a .state
// exactly as Simulation's constructor and run() do before the first step:
// SerialCalcs::createBox -> loadBoxData (FileUtilities.cpp:19-168), then
// Box::keepMoleculeInBox for every molecule (Simulation.cpp:70-72) and
// SimBoxBuilder::build (Simulation.cpp:118-121).  Returns 0 on success and
// the counts of the built SimBox.
int ref_load(const char* path, int* n_mol, int* n_atom, int* n_pidx, long* start_step,
             long* steps) {
  SimulationArgs args = SimulationArgs();
  args.filePath = path;
  std::string p(path);
  const std::string ext = p.substr(p.find_last_of('.') + 1);
  args.fileType = ext == "config" ? InputFile::Configuration
                : ext == "state"  ? InputFile::State
                                  : InputFile::Unknown;
  args.strategy = Strategy::Default;
  SBScanner* sbs = new SBScanner();
  long st = 0, n = 0;
  Box* box = SerialCalcs::createBox(args, &st, &n, sbs);
  if (!box) return 1;
  for (int m = 0; m < box->environment->numOfMolecules; m++) box->keepMoleculeInBox(m);
  SimBoxBuilder builder = SimBoxBuilder(false, sbs);
  g_lbox = box;
  g_lsb = builder.build(box);
  g_lstart = st;
  g_lsteps = n;
  *n_mol = g_lsb->numMolecules;
  *n_atom = g_lsb->numAtoms;
  *n_pidx = g_lsb->numPIdxes;
  *start_step = st;
  *steps = n;
  return 0;
}

// The loaded SimBox rows (SimBox.h:120-149): coordinates, sigma/epsilon/
// charge, molecule start/length/type/primary range, primary indexes, box
// edges and [cutoff, temperature, kT, max translation, max rotation].
void ref_load_rows(double* x, double* y, double* z, double* sigma, double* epsilon,
                   double* charge, int* mol_start, int* mol_len, int* mol_type,
                   int* mol_pidx_start, int* mol_pidx_count, int* pidx, double* size,
                   double* params) {
  SimBox* sb = g_lsb;
  const int na = sb->numAtoms, nm = sb->numMolecules;
  std::memcpy(x, sb->atomCoordinates[X_COORD], sizeof(double) * na);
  std::memcpy(y, sb->atomCoordinates[Y_COORD], sizeof(double) * na);
  std::memcpy(z, sb->atomCoordinates[Z_COORD], sizeof(double) * na);
  std::memcpy(sigma, sb->atomData[ATOM_SIGMA], sizeof(double) * na);
  std::memcpy(epsilon, sb->atomData[ATOM_EPSILON], sizeof(double) * na);
  std::memcpy(charge, sb->atomData[ATOM_CHARGE], sizeof(double) * na);
  std::memcpy(mol_start, sb->moleculeData[MOL_START], sizeof(int) * nm);
  std::memcpy(mol_len, sb->moleculeData[MOL_LEN], sizeof(int) * nm);
  std::memcpy(mol_type, sb->moleculeData[MOL_TYPE], sizeof(int) * nm);
  std::memcpy(mol_pidx_start, sb->moleculeData[MOL_PIDX_START], sizeof(int) * nm);
  std::memcpy(mol_pidx_count, sb->moleculeData[MOL_PIDX_COUNT], sizeof(int) * nm);
  std::memcpy(pidx, sb->primaryIndexes, sizeof(int) * sb->numPIdxes);
  std::memcpy(size, sb->size, sizeof(double) * 3);
  params[0] = sb->cutoff;
  params[1] = sb->temperature;
  params[2] = sb->kT;
  params[3] = sb->maxTranslate;
  params[4] = sb->maxRotate;
}

// SerialCalcs::calcEnergy_LRC of the loaded box (SerialCalcs.cpp:37-107).
double ref_load_lrc(void) { return SerialCalcs::calcEnergy_LRC(g_lbox); }

// The loaded environment's seed (Simulation.cpp:45-50 seeds the RNG with it).
int ref_load_seed(void) { return g_lbox->environment->randomseed; }

// Sets the loaded SimBox's coordinates (e.g. to those of a trajectory the
// harness ran on a SimBox with the same rows).
void ref_load_set_coords(const double* x, const double* y, const double* z) {
  const int na = g_lsb->numAtoms;
  std::memcpy(g_lsb->atomCoordinates[X_COORD], x, sizeof(double) * na);
  std::memcpy(g_lsb->atomCoordinates[Y_COORD], y, sizeof(double) * na);
  std::memcpy(g_lsb->atomCoordinates[Z_COORD], z, sizeof(double) * na);
}

// StateScanner::outputState of the loaded box at the loaded SimBox
// coordinates (Simulation.cpp:353-375).
void ref_load_write_state(const char* path, int step) {
  StateScanner ss = StateScanner("");
  ss.outputState(g_lbox->getEnvironment(), g_lbox->getMolecules(), g_lbox->getMoleculeCount(),
                 step, path, g_lsb->atomCoordinates);
}

// ---- flexible molecules (the reference's intramolecular code) -----------------------
//
// The reference compiles its bond / angle code but gates its three call sites
// with ENABLE_INTRA (SimulationStep.h:15, false): calcMoleculeEnergy adds
// calcIntraMolecularEnergy (SimulationStep.cpp:15-18), changeMolecule follows
// intermolecularMove with intramolecularMove (:424-428), and rollback also
// restores the angle sizes and bond lengths (:745-748).  The functions below
// call the reference's own SimCalcs functions and compose them at exactly
// those three sites, i.e. the reference as it runs with ENABLE_INTRA true.

// Makes the SimBox built by ref_load the one every other harness function
// acts on (its step object, SimCalcs::sb and the GPUCopy host rows).
void ref_load_activate(void) {
  g_sb = g_lsb;
  GPUCopy::setParallel(false);
  GPUCopy::copyIn(g_sb);
  delete g_step;
  g_step = new BruteForceStep(g_sb);
}

void ref_topology_counts(int* n_bond, int* n_angle, int* n_mol) {
  *n_bond = g_sb->numBonds;
  *n_angle = g_sb->numAngles;
  *n_mol = g_sb->numMolecules;
}

// The bond and angle rows, per-molecule ranges and type, and
// params = [maxBondDelta, maxAngleDelta, maxIntraMoves, hasFlexibleBonds,
// hasFlexibleAngles, stepNum].
void ref_topology_rows(int* bond_a1, int* bond_a2, double* bond_k, double* bond_eq,
                       double* bond_len, int* bond_var, int* angle_a1, int* angle_a2,
                       int* angle_mid, double* angle_k, double* angle_eq, double* angle_size,
                       int* angle_var, int* mol_bond_start, int* mol_bond_count,
                       int* mol_angle_start, int* mol_angle_count, int* mol_type,
                       double* params) {
  SimBox* sb = g_sb;
  for (int i = 0; i < sb->numBonds; i++) {
    bond_a1[i] = (int)sb->bondData[BOND_A1_IDX][i];
    bond_a2[i] = (int)sb->bondData[BOND_A2_IDX][i];
    bond_k[i] = sb->bondData[BOND_KBOND][i];
    bond_eq[i] = sb->bondData[BOND_EQDIST][i];
    bond_len[i] = sb->bondLengths[i];
    bond_var[i] = (int)sb->bondData[BOND_VARIABLE][i];
  }
  for (int i = 0; i < sb->numAngles; i++) {
    angle_a1[i] = (int)sb->angleData[ANGLE_A1_IDX][i];
    angle_a2[i] = (int)sb->angleData[ANGLE_A2_IDX][i];
    angle_mid[i] = (int)sb->angleData[ANGLE_MID_IDX][i];
    angle_k[i] = sb->angleData[ANGLE_KANGLE][i];
    angle_eq[i] = sb->angleData[ANGLE_EQANGLE][i];
    angle_size[i] = sb->angleSizes[i];
    angle_var[i] = (int)sb->angleData[ANGLE_VARIABLE][i];
  }
  for (int m = 0; m < sb->numMolecules; m++) {
    mol_bond_start[m] = sb->moleculeData[MOL_BOND_START][m];
    mol_bond_count[m] = sb->moleculeData[MOL_BOND_COUNT][m];
    mol_angle_start[m] = sb->moleculeData[MOL_ANGLE_START][m];
    mol_angle_count[m] = sb->moleculeData[MOL_ANGLE_COUNT][m];
    mol_type[m] = sb->moleculeData[MOL_TYPE][m];
  }
  params[0] = sb->maxBondDelta;
  params[1] = sb->maxAngleDelta;
  params[2] = sb->maxIntraMoves;
  params[3] = sb->hasFlexibleBonds ? 1 : 0;
  params[4] = sb->hasFlexibleAngles ? 1 : 0;
  params[5] = sb->stepNum;
}

// Type t's intramolecular pair factors as calcIntraMolecularEnergy finds them
// in the exclusion and fudge lists (SimulationStep.cpp:95-117): out[i*n + j]
// = 0 (excluded), 1 (fudge 0.5) or 2 (full), for i != j.  Returns 1 when
// the type has no lists.
int ref_type_codes(int t, int n, unsigned char* out) {
  if (!g_sb->excludeAtoms || !g_sb->excludeAtoms[t]) return 1;
  for (int i = 0; i < n; i++) {
    for (int j = 0; j < n; j++) {
      unsigned char c = 2;
      for (int k = 0;; k++) {
        int v = g_sb->excludeAtoms[t][i][k];
        if (v == -1) break;
        if (v == j) { c = 0; break; }
      }
      if (c) {
        for (int k = 0;; k++) {
          int v = g_sb->fudgeAtoms[t][i][k];
          if (v == -1) break;
          if (v == j) { c = 1; break; }
        }
      }
      out[i * n + j] = c;
    }
  }
  return 0;
}

// Replaces the current SimBox's bond and angle rows, per-molecule ranges and
// types, exclusion and fudge lists (from per-type codes as above, natom[t]
// atoms each, matrices concatenated) and the intramolecular settings, the
// way SimBoxBuilder.cpp:44-278 leaves them.
void ref_set_topology(int n_bond, const int* bond_a1, const int* bond_a2, const double* bond_k,
                      const double* bond_eq, const double* bond_len, const int* bond_var,
                      int n_angle, const int* angle_a1, const int* angle_a2,
                      const int* angle_mid, const double* angle_k, const double* angle_eq,
                      const double* angle_size, const int* angle_var,
                      const int* mol_bond_start, const int* mol_bond_count,
                      const int* mol_angle_start, const int* mol_angle_count,
                      const int* mol_type, int n_type, const int* natom,
                      const unsigned char* codes, double max_bond_delta,
                      double max_angle_delta, int max_intra_moves, int step_num) {
  SimBox* sb = g_sb;
  sb->numBonds = n_bond;
  sb->numAngles = n_angle;
  sb->bondData = new Real*[BOND_DATA_SIZE];
  for (int r = 0; r < BOND_DATA_SIZE; r++) sb->bondData[r] = new Real[n_bond > 0 ? n_bond : 1];
  sb->bondLengths = new Real[n_bond > 0 ? n_bond : 1];
  sb->rollBackBondLengths = new Real[n_bond > 0 ? n_bond : 1];
  sb->hasFlexibleBonds = false;
  for (int i = 0; i < n_bond; i++) {
    sb->bondData[BOND_A1_IDX][i] = bond_a1[i];
    sb->bondData[BOND_A2_IDX][i] = bond_a2[i];
    sb->bondData[BOND_KBOND][i] = bond_k[i];
    sb->bondData[BOND_EQDIST][i] = bond_eq[i];
    sb->bondData[BOND_VARIABLE][i] = bond_var[i];
    sb->bondLengths[i] = bond_len[i];
    sb->rollBackBondLengths[i] = 0;
    sb->hasFlexibleBonds |= bond_var[i] != 0;
  }
  sb->angleData = new Real*[ANGLE_DATA_SIZE];
  for (int r = 0; r < ANGLE_DATA_SIZE; r++) sb->angleData[r] = new Real[n_angle > 0 ? n_angle : 1];
  sb->angleSizes = new Real[n_angle > 0 ? n_angle : 1];
  sb->rollBackAngleSizes = new Real[n_angle > 0 ? n_angle : 1];
  sb->hasFlexibleAngles = false;
  for (int i = 0; i < n_angle; i++) {
    sb->angleData[ANGLE_A1_IDX][i] = angle_a1[i];
    sb->angleData[ANGLE_A2_IDX][i] = angle_a2[i];
    sb->angleData[ANGLE_MID_IDX][i] = angle_mid[i];
    sb->angleData[ANGLE_KANGLE][i] = angle_k[i];
    sb->angleData[ANGLE_EQANGLE][i] = angle_eq[i];
    sb->angleData[ANGLE_VARIABLE][i] = angle_var[i];
    sb->angleSizes[i] = angle_size[i];
    sb->rollBackAngleSizes[i] = 0;
    sb->hasFlexibleAngles |= angle_var[i] != 0;
  }
  for (int m = 0; m < sb->numMolecules; m++) {
    sb->moleculeData[MOL_BOND_START][m] = mol_bond_start[m];
    sb->moleculeData[MOL_BOND_COUNT][m] = mol_bond_count[m];
    sb->moleculeData[MOL_ANGLE_START][m] = mol_angle_start[m];
    sb->moleculeData[MOL_ANGLE_COUNT][m] = mol_angle_count[m];
    sb->moleculeData[MOL_TYPE][m] = mol_type[m];
  }
  sb->excludeAtoms = new int**[n_type > 0 ? n_type : 1];
  sb->fudgeAtoms = new int**[n_type > 0 ? n_type : 1];
  const unsigned char* c = codes;
  for (int t = 0; t < n_type; t++) {
    const int n = natom[t];
    sb->excludeAtoms[t] = n > 0 ? new int*[n] : NULL;
    sb->fudgeAtoms[t] = n > 0 ? new int*[n] : NULL;
    for (int i = 0; i < n; i++) {
      int ne = 0, nf = 0;
      for (int j = 0; j < n; j++) {
        ne += c[i * n + j] == 0;
        nf += c[i * n + j] == 1;
      }
      int* e = new int[ne + 1];
      int* f = new int[nf + 1];
      ne = nf = 0;
      for (int j = 0; j < n; j++) {
        if (c[i * n + j] == 0) e[ne++] = j;
        if (c[i * n + j] == 1) f[nf++] = j;
      }
      e[ne] = -1;
      f[nf] = -1;
      sb->excludeAtoms[t][i] = e;
      sb->fudgeAtoms[t][i] = f;
    }
    c += (size_t)n * n;
  }
  sb->maxBondDelta = max_bond_delta;
  sb->maxAngleDelta = max_angle_delta;
  sb->maxIntraMoves = max_intra_moves;
  sb->stepNum = step_num;
  sb->numBondMoves = sb->numAcceptedBondMoves = 0;
  sb->numAngleMoves = sb->numAcceptedAngleMoves = 0;
  GPUCopy::copyIn(sb);
}

// SimCalcs::calcIntraMolecularEnergy, bondEnergy, angleEnergy
// (SimulationStep.cpp:80-146, :241-255).
double ref_intra_energy(int mol) { return SimCalcs::calcIntraMolecularEnergy(mol); }
double ref_bond_energy(int mol) { return SimCalcs::bondEnergy(mol); }
double ref_angle_energy(int mol) { return SimCalcs::angleEnergy(mol); }

// SimCalcs::stretchBond (:257-315) and SimCalcs::expandAngle (:148-239).
void ref_stretch_bond(int mol, int bond, double dist) { SimCalcs::stretchBond(mol, bond, dist); }
void ref_expand_angle(int mol, int angle, double deg) { SimCalcs::expandAngle(mol, angle, deg); }

// SimCalcs::saveBonds / saveAngles (:677-701).
void ref_save_intra(int mol) {
  SimCalcs::saveBonds(mol);
  SimCalcs::saveAngles(mol);
}

// SimCalcs::intramolecularMove (:568-675), drawing from rand().
void ref_intramolecular_move(int mol) { SimCalcs::intramolecularMove(mol); }

// SimCalcs::rollback with its ENABLE_INTRA branch (:731-749).
void ref_intra_rollback(int mol) {
  SimCalcs::rollback(mol);
  SimCalcs::rollbackAngles(mol);
  SimCalcs::rollbackBonds(mol);
}

// SimulationStep::calcMoleculeEnergy with ENABLE_INTRA (SimulationStep.cpp:15-18).
double ref_mol_energy_intra(int curr, int start) {
  return g_step->calcMolecularEnergyContribution(curr, start) +
         SimCalcs::calcIntraMolecularEnergy(curr);
}

// SimulationStep::calcSystemEnergy with ENABLE_INTRA (:40-71, VERBOSE output
// left out).
double ref_system_energy_intra(void) {
  Real total = 0;
  for (int mol = 0; mol < g_sb->numMolecules; mol++) total += ref_mol_energy_intra(mol, mol);
  return total;
}

// The bond lengths, angle sizes and
// out = [maxBondDelta, maxAngleDelta, stepNum, numBondMoves,
// numAcceptedBondMoves, numAngleMoves, numAcceptedAngleMoves].
void ref_intra_state(double* bond_len, double* angle_size, double* out) {
  std::memcpy(bond_len, g_sb->bondLengths, sizeof(double) * g_sb->numBonds);
  std::memcpy(angle_size, g_sb->angleSizes, sizeof(double) * g_sb->numAngles);
  out[0] = g_sb->maxBondDelta;
  out[1] = g_sb->maxAngleDelta;
  out[2] = g_sb->stepNum;
  out[3] = g_sb->numBondMoves;
  out[4] = g_sb->numAcceptedBondMoves;
  out[5] = g_sb->numAngleMoves;
  out[6] = g_sb->numAcceptedAngleMoves;
}

void ref_set_step(int step) { g_sb->stepNum = step; }

// Simulation::run's NVT loop (Simulation.cpp:219-264) as it runs with
// ENABLE_INTRA true: molecule energies with the intramolecular term, the
// intramolecular move after the rigid one, rollbacks restoring angles and
// bonds, the step counter the tuning reads.
double ref_run_plain_intra(int steps, double e0, int* accepted) {
  double e = e0;
  int acc = 0;
  for (int move = 0; move < steps; move++) {
    int idx = g_step->chooseMolecule(g_sb);
    double old_e = ref_mol_energy_intra(idx, 0);
    SimCalcs::intermolecularMove(idx);
    SimCalcs::intramolecularMove(idx);
    double new_e = ref_mol_energy_intra(idx, 0);
    if (SimCalcs::acceptMove(new_e - old_e)) {
      acc++;
      e += new_e - old_e;
    } else {
      ref_intra_rollback(idx);
    }
    g_sb->stepNum++;
  }
  if (accepted) *accepted = acc;
  return e;
}

}  // extern "C"
