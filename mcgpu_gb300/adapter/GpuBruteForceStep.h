// GpuBruteForceStep.h -- the reference-side binding: a SimulationStep
// (src/Metropolis/SimulationStep.h:24-94) whose four virtual members run on
// the GB300 through the C ABI of libmcgpu_gb300.so.  Compiled against the
// reference's own headers; Simulation::run constructs it where it constructs
// BruteForceStep (src/Metropolis/Simulation.cpp:141-157).
#ifndef MCGPU_GB300_GPU_BRUTE_FORCE_STEP_H
#define MCGPU_GB300_GPU_BRUTE_FORCE_STEP_H

#include "Metropolis/SimulationStep.h"
#include "mcgpu_gb300.h"

class GpuBruteForceStep : public SimulationStep {
 public:
  // Uploads the SimBox rows to the GPU (replaces GPUCopy::copyIn).
  // precision: MCGPU_PREC_FP64 (the reference's Real=double arithmetic) or
  // MCGPU_PREC_MIXED (FP32 pair terms, FP64 sums).
  // intra: the reference's intramolecular moves on the GPU (what its
  // ENABLE_INTRA, SimulationStep.h:15, turns on in its own code): the SimBox's
  // bond / angle rows and exclusion lists are uploaded, molecule energies
  // carry the intramolecular term and changeMolecule makes the
  // intramolecular move.  Build the reference with ENABLE_INTRA false when
  // using it, so that SimulationStep::calcMoleculeEnergy does not add the
  // host's own intramolecular term on top.
  explicit GpuBruteForceStep(SimBox* box, int precision = MCGPU_PREC_FP64, int device = 0,
                             bool intra = false);
  ~GpuBruteForceStep();

  // BruteForceCalcs::calcMolecularEnergyContribution (BruteForceStep.cpp:15-46).
  Real calcMolecularEnergyContribution(int currMol, int startMol) override;
  // SimCalcs::intermolecularMove (SimulationStep.cpp:520-566): the seven draws
  // come from the reference's randomReal in its order; the move runs on the
  // GPU.  With intra, then SimCalcs::intramolecularMove (:568-675) on the GPU,
  // its draws from the same rand(), the tuning reading box->stepNum.
  void changeMolecule(int molIdx, SimBox* box) override;
  // SimCalcs::rollback (SimulationStep.cpp:731-749).
  void rollback(int molIdx, SimBox* box) override;
  // SimulationStep::calcSystemEnergy (SimulationStep.cpp:40-71).
  Real calcSystemEnergy(Real& subLJ, Real& subCharge, int numMolecules) override;

  // Copies the device coordinates back into the SimBox rows (replaces
  // GPUCopy::copyOut) before saveState / writePDB read them.
  void copyOut(SimBox* box);

 private:
  void check(int status, const char* what);
  void uploadTopology(SimBox* box);
  mcgpu_ctx* ctx_ = nullptr;
  mcgpu_box* gbox_ = nullptr;
  bool intra_ = false;
};

#endif
