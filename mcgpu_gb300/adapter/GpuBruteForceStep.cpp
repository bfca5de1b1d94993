// GpuBruteForceStep.cpp -- see GpuBruteForceStep.h.
#include "GpuBruteForceStep.h"

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "Metropolis/Utilities/MathLibrary.h"

void GpuBruteForceStep::check(int status, const char* what) {
  if (status == MCGPU_OK) return;
  char msg[512];
  mcgpu_last_error(ctx_, msg, sizeof(msg));
  std::fprintf(stderr, "GpuBruteForceStep: %s failed (%d): %s\n", what, status, msg);
  std::exit(EXIT_FAILURE);  // the reference's own error behaviour (Simulation.cpp:48)
}

GpuBruteForceStep::GpuBruteForceStep(SimBox* sb, int precision, int device)
    : SimulationStep(sb) {
  check(mcgpu_ctx_create(&ctx_, device), "mcgpu_ctx_create");
  mcgpu_box_desc d = {};
  d.n_mol = sb->numMolecules;
  d.n_atom = sb->numAtoms;
  d.n_pidx = sb->numPIdxes;
  d.x = sb->atomCoordinates[X_COORD];
  d.y = sb->atomCoordinates[Y_COORD];
  d.z = sb->atomCoordinates[Z_COORD];
  d.sigma = sb->atomData[ATOM_SIGMA];
  d.epsilon = sb->atomData[ATOM_EPSILON];
  d.charge = sb->atomData[ATOM_CHARGE];
  d.mol_start = sb->moleculeData[MOL_START];
  d.mol_len = sb->moleculeData[MOL_LEN];
  d.mol_pidx_start = sb->moleculeData[MOL_PIDX_START];
  d.mol_pidx_count = sb->moleculeData[MOL_PIDX_COUNT];
  d.pidx = sb->primaryIndexes;
  for (int k = 0; k < 3; k++) d.size[k] = sb->size[k];
  d.cutoff = sb->cutoff;
  d.temperature = sb->temperature;
  d.max_translate = sb->maxTranslate;
  d.max_rotate = sb->maxRotate;
  check(mcgpu_box_upload(ctx_, &d, precision, &gbox_), "mcgpu_box_upload");
}

GpuBruteForceStep::~GpuBruteForceStep() {
  mcgpu_box_destroy(gbox_);
  mcgpu_ctx_destroy(ctx_);
}

Real GpuBruteForceStep::calcMolecularEnergyContribution(int currMol, int startMol) {
  double e = 0;
  check(mcgpu_mol_energy(gbox_, currMol, startMol, &e), "mcgpu_mol_energy");
  return e;
}

void GpuBruteForceStep::changeMolecule(int molIdx, SimBox* sb) {
  const Real maxT = sb->maxTranslate, maxR = sb->maxRotate;
  const int molLen = sb->moleculeData[MOL_LEN][molIdx];
  mcgpu_move mv = {};
  mv.vertex = (int)randomReal(0, molLen);
  if (mv.vertex >= molLen) mv.vertex = molLen - 1;  // rand() == RAND_MAX
  mv.dx = randomReal(-maxT, maxT);
  mv.dy = randomReal(-maxT, maxT);
  mv.dz = randomReal(-maxT, maxT);
  mv.rx = randomReal(-maxR, maxR);
  mv.ry = randomReal(-maxR, maxR);
  mv.rz = randomReal(-maxR, maxR);
  check(mcgpu_change_molecule(gbox_, molIdx, &mv), "mcgpu_change_molecule");
}

void GpuBruteForceStep::rollback(int molIdx, SimBox* sb) {
  check(mcgpu_rollback(gbox_, molIdx), "mcgpu_rollback");
}

Real GpuBruteForceStep::calcSystemEnergy(Real& subLJ, Real& subCharge, int numMolecules) {
  double e = 0;
  check(mcgpu_system_energy(gbox_, &e), "mcgpu_system_energy");
  return e + subLJ + subCharge;
}

void GpuBruteForceStep::copyOut(SimBox* sb) {
  check(mcgpu_box_download(gbox_, sb->atomCoordinates[X_COORD], sb->atomCoordinates[Y_COORD],
                           sb->atomCoordinates[Z_COORD], sb->size),
        "mcgpu_box_download");
}
