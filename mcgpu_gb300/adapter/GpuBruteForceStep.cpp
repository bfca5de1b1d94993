// GpuBruteForceStep.cpp -- see GpuBruteForceStep.h.
#include "GpuBruteForceStep.h"

#include <algorithm>
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

GpuBruteForceStep::GpuBruteForceStep(SimBox* sb, int precision, int device, bool intra)
    : SimulationStep(sb), intra_(intra) {
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
  if (intra_) {
    uploadTopology(sb);
    check(mcgpu_box_set_intra(gbox_, 1), "mcgpu_box_set_intra");
  }
}

// The SimBox's bond / angle rows (SimBox.h:160-221, Real rows holding
// indexes and flags) and exclusion / fudge lists (SimBox.h:298-305, one list
// set per molecule type, sized by the type's first molecule) as the C ABI's
// integer rows and per-type pair codes.
void GpuBruteForceStep::uploadTopology(SimBox* sb) {
  const int nb = sb->numBonds, na = sb->numAngles, nm = sb->numMolecules;
  std::vector<int> ba1(nb), ba2(nb), bvar(nb), aa1(na), aa2(na), amid(na), avar(na);
  for (int i = 0; i < nb; i++) {
    ba1[i] = (int)sb->bondData[BOND_A1_IDX][i];
    ba2[i] = (int)sb->bondData[BOND_A2_IDX][i];
    bvar[i] = sb->bondData[BOND_VARIABLE][i] != 0;
  }
  for (int i = 0; i < na; i++) {
    aa1[i] = (int)sb->angleData[ANGLE_A1_IDX][i];
    aa2[i] = (int)sb->angleData[ANGLE_A2_IDX][i];
    amid[i] = (int)sb->angleData[ANGLE_MID_IDX][i];
    avar[i] = sb->angleData[ANGLE_VARIABLE][i] != 0;
  }
  int n_type = 0;
  for (int m = 0; m < nm; m++) n_type = std::max(n_type, sb->moleculeData[MOL_TYPE][m] + 1);
  std::vector<int> natom(n_type, 0);
  for (int m = nm - 1; m >= 0; m--) natom[sb->moleculeData[MOL_TYPE][m]] = sb->moleculeData[MOL_LEN][m];
  std::vector<unsigned char> codes;
  for (int t = 0; t < n_type; t++) {
    const int n = natom[t];
    for (int i = 0; i < n; i++) {
      for (int j = 0; j < n; j++) {
        unsigned char c = 2;
        for (int k = 0; sb->excludeAtoms && sb->excludeAtoms[t]; k++) {
          const int v = sb->excludeAtoms[t][i][k];
          if (v == -1) break;
          if (v == j) { c = 0; break; }
        }
        for (int k = 0; c && sb->fudgeAtoms && sb->fudgeAtoms[t]; k++) {
          const int v = sb->fudgeAtoms[t][i][k];
          if (v == -1) break;
          if (v == j) { c = 1; break; }
        }
        codes.push_back(c);
      }
    }
  }
  mcgpu_topology_desc t = {};
  t.n_bond = nb;
  t.n_angle = na;
  t.n_type = n_type;
  t.max_intra_moves = sb->maxIntraMoves;
  t.bond_a1 = ba1.data();
  t.bond_a2 = ba2.data();
  t.bond_var = bvar.data();
  t.bond_k = sb->bondData[BOND_KBOND];
  t.bond_eq = sb->bondData[BOND_EQDIST];
  t.bond_len = sb->bondLengths;
  t.angle_a1 = aa1.data();
  t.angle_a2 = aa2.data();
  t.angle_mid = amid.data();
  t.angle_var = avar.data();
  t.angle_k = sb->angleData[ANGLE_KANGLE];
  t.angle_eq = sb->angleData[ANGLE_EQANGLE];
  t.angle_size = sb->angleSizes;
  t.mol_bond_start = sb->moleculeData[MOL_BOND_START];
  t.mol_bond_count = sb->moleculeData[MOL_BOND_COUNT];
  t.mol_angle_start = sb->moleculeData[MOL_ANGLE_START];
  t.mol_angle_count = sb->moleculeData[MOL_ANGLE_COUNT];
  t.mol_type = sb->moleculeData[MOL_TYPE];
  t.type_natom = natom.data();
  t.pair_code = codes.data();
  t.max_bond_delta = sb->maxBondDelta;
  t.max_angle_delta = sb->maxAngleDelta;
  t.step_num = sb->stepNum;
  check(mcgpu_box_set_topology(gbox_, &t), "mcgpu_box_set_topology");
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
  if (intra_) check(mcgpu_intra_set_step(gbox_, sb->stepNum), "mcgpu_intra_set_step");
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
