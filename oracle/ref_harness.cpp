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

}  // extern "C"
