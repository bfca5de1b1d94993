// intra.h -- flexible molecules on the plain path: the bond / angle rows on
// the device, the host's copy of what the draws need, and the launchers of
// intra.cu (the intramolecular energy, bond stretches and angle expansions,
// the rollback of the rows).
#pragma once

#include <memory>
#include <vector>

#include "crand.h"
#include "host.h"
#include "mcgpu_gb300.h"

namespace mcgpu {

// Stretches or expansions one launch applies (maxIntraMoves is 15 in the
// reference; longer lists go in several launches).
constexpr int kIntraOps = 16;

enum : int { kIntraSave = 1, kIntraEnergyBefore = 2, kIntraEnergyAfter = 4 };

// Device view of the rows.  Bond and angle rows are indexed as the
// reference's (box-absolute), molecules by their box index.  Per bond and
// angle the host precomputes the partition the reference's union-find finds
// on every call (it depends on the bonds only): part_off < 0 marks a bond in
// a ring or an angle whose ends share a component (the call changes
// nothing); otherwise part[part_off + i] for atom i of the molecule is 1 for
// the side that moves +d/2 (a bond's second end) or the first end's group
// (turns by -deg), 2 for the second end's group (+deg), 0 otherwise.
struct IntraRows {
  int n_bond, n_angle, flex_bonds, flex_angles;
  const int *b_a1, *b_a2, *b_var, *b_part;
  const double *b_k, *b_eq;
  double *b_len, *b_len_rb;
  const int *a_a1, *a_a2, *a_mid, *a_var, *a_part;
  const double *a_k, *a_eq;
  double *a_size, *a_size_rb;
  const int *m_bstart, *m_bcount, *m_astart, *m_acount, *m_type;
  const int *t_natom, *t_off;
  const unsigned char *code, *part;
};

// One launch's stretches (kind 0) or expansions (kind 1) of molecule mol,
// in order; for an expansion the cosines and sines of the two groups'
// angles (deg * -DEG2RAD and deg * DEG2RAD), taken on the host by the C
// library as the reference takes them.
struct IntraOps {
  int mol, kind, n, flags;
  int idx[kIntraOps];
  double amt[kIntraOps];
  double c1[kIntraOps], s1[kIntraOps], c2[kIntraOps], s2[kIntraOps];
};

struct IntraHost {
  IntraRows R{};
  std::vector<void*> allocs;
  int n_bond = 0, n_angle = 0, n_type = 0, max_intra_moves = 15;
  std::vector<int> bstart, bcount, astart, acount, bvar, avar;
  bool flex_bonds = false, flex_angles = false;
  double max_bond_delta = 0, max_angle_delta = 0;
  long long step = 0, bond_moves = 0, bond_accepted = 0, angle_moves = 0, angle_accepted = 0;
  double* dout = nullptr;   // device [2]: energy before / after a stage
  double* hout = nullptr;   // pinned [2]
  ~IntraHost();
};

// Validates the topology against the box (n_mol molecules, n_atom atoms,
// molecule starts / lengths) and uploads it; the rollback rows start equal
// to the rows.
int intra_upload(mcgpu_ctx* ctx, int n_mol, int n_atom, const int* mol_start,
                 const int* mol_len, const mcgpu_topology_desc* t,
                 std::unique_ptr<IntraHost>* out);

// out[0] = calcIntraMolecularEnergy(mol) of chain `chain`'s molecule mol.
cudaError_t launch_intra_energy(const Pool& P, const IntraRows& R, int chain, int mol,
                                double* out, cudaStream_t st);
// The stage ops.mol: save rows (kIntraSave), out[0] = energy before
// (kIntraEnergyBefore), the ops, the molecule's mirrors, out[1] = energy
// after (kIntraEnergyAfter).
cudaError_t launch_intra_ops(const Pool& P, const IntraRows& R, int chain, const IntraOps& ops,
                             double* out, cudaStream_t st);
// SimCalcs::rollback with its ENABLE_INTRA branch: coordinates from the
// rollback copy, angle sizes and bond lengths from theirs, mirrors.
cudaError_t launch_intra_rollback(const Pool& P, const IntraRows& R, int chain, int mol,
                                  cudaStream_t st);
// emol[m] += calcIntraMolecularEnergy(m) for the n_mol molecules of chain 0
// (the intramolecular terms of calcSystemEnergy).
cudaError_t launch_intra_add(const Pool& P, const IntraRows& R, int n_mol, double* emol,
                             cudaStream_t st);

// Most bonds or angles one stage of the device loop moves (max_intra_moves).
constexpr int kLoopSel = 64;

// State of the device-resident run of the reference's loop (kept in device
// memory between launches): the C library's generator, the running energy,
// the counters, and the intramolecular widths, step counter and tuning
// counters.  error: 1 when a stage's index draws did not fill its set within
// kLoopDrawCap draws (the loop stops).
struct PlainLoop {
  CRand rng;
  double energy;
  long long accepted, rejected, pairs;
  long long step;
  double max_bond_delta, max_angle_delta;
  long long bond_moves, bond_accepted, angle_moves, angle_accepted;
  int max_intra_moves, error;
};

// One box of a device loop launch: its pool (chain 0), bond / angle rows
// (when intra != 0) and loop state.
struct LoopTask {
  Pool P;
  IntraRows R;
  PlainLoop* L;
  int intra, pad;
};

// n_steps of Simulation::run's loop for each of n_tasks boxes, one CTA per
// box, the draws from each L->rng; intra != 0: with the intramolecular term
// and move.  f64: FP64 intermolecular pair terms, else FP32.  tasks is a
// device array.
cudaError_t launch_plain_steps(bool f64, const LoopTask* tasks, int n_tasks, int n_steps,
                               SmemShape sh, cudaStream_t st);

}  // namespace mcgpu
