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
  explicit GpuBruteForceStep(SimBox* box, int precision = MCGPU_PREC_FP64, int device = 0);
  ~GpuBruteForceStep();

  // BruteForceCalcs::calcMolecularEnergyContribution (BruteForceStep.cpp:15-46).
  Real calcMolecularEnergyContribution(int currMol, int startMol) override;
  // SimCalcs::intermolecularMove (SimulationStep.cpp:520-566): the seven draws
  // come from the reference's randomReal in its order; the move runs on the GPU.
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
  mcgpu_ctx* ctx_ = nullptr;
  mcgpu_box* gbox_ = nullptr;
};

#endif
