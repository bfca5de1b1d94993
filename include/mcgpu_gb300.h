/*
 * mcgpu_gb300.h -- C ABI of the GB300-native Metropolis trial-move energy
 * path.  Plain pointers and sizes only; every call returns an mcgpu_status
 * (0 = ok) and leaves a message for mcgpu_last_error() on failure.
 *
 * The plain single-chain entry points replace, one for one, the
 * SimulationStep contract that MCGPU's Simulation::run drives
 * (src/Metropolis/SimulationStep.h:24-94) over the SimBox rows
 * (src/Metropolis/SimBox.h:120-149) that GPUCopy mirrors to the device
 * (src/Metropolis/GPUCopy.cpp:97-188).  The chain, batch and serve entry
 * points are the device-resident forms: the proposal RNG, the energy
 * difference, the Metropolis decision and the commit or rollback all stay on
 * the GPU.
 *
 * Thread safety: a context and the boxes, batches and servers made from it
 * belong to one host thread at a time.
 */
#ifndef MCGPU_GB300_H
#define MCGPU_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  MCGPU_OK = 0,
  MCGPU_ERR_INVALID = 1,     /* bad argument (index, size, null pointer)   */
  MCGPU_ERR_CUDA = 2,        /* a CUDA runtime call failed                 */
  MCGPU_ERR_NOMEM = 3,       /* device or host allocation failed           */
  MCGPU_ERR_UNSUPPORTED = 4, /* outside the supported limits (see below)   */
  MCGPU_ERR_DEVICE = 5,      /* a kernel reported an error status word     */
  MCGPU_ERR_CAPACITY = 6     /* server slot table or HBM budget exhausted  */
} mcgpu_status;

/* Pair arithmetic of a box. */
typedef enum {
  MCGPU_PREC_FP64 = 0,  /* FP64 pair terms, the reference's Real=double     */
  MCGPU_PREC_MIXED = 1  /* FP32 pair terms, FP64 per-neighbour sums and totals */
} mcgpu_precision;

/* Rotation form of a device-drawn trial move. */
typedef enum {
  MCGPU_ROT_EULER = 0,  /* X->Y->Z Euler angles in degrees about the vertex atom
                           (SimulationStep.cpp:527-555)                     */
  MCGPU_ROT_AXIS = 1    /* angle about a uniform random axis through the vertex */
} mcgpu_rotation;

/* Limits of this build. */
#define MCGPU_MAX_MOL_ATOMS 64   /* atoms in one molecule                      */
#define MCGPU_MAX_MOL_PIDX 8     /* primary indexes of one molecule            */

/* Host description of one box: the SimBox rows, FP64, structure of arrays.
 * mol_pidx_* index into pidx[], and pidx[] holds absolute atom indexes, as
 * SimBoxBuilder::addPrimaryIndexes builds them (SimBoxBuilder.cpp:282-299). */
typedef struct {
  int32_t n_mol, n_atom, n_pidx, pad0;
  const double *x, *y, *z;             /* atomCoordinates rows [n_atom]     */
  const double *sigma, *epsilon, *charge; /* atomData rows [n_atom]         */
  const int32_t *mol_start, *mol_len;  /* moleculeData MOL_START / MOL_LEN  */
  const int32_t *mol_pidx_start, *mol_pidx_count; /* MOL_PIDX_START/COUNT   */
  const int32_t *pidx;                 /* primaryIndexes [n_pidx]           */
  double size[3];                      /* box edges (cubic in practice)     */
  double cutoff;                       /* molecular cutoff, Angstrom        */
  double temperature;                  /* K; kT = T * 0.00198717            */
  double max_translate, max_rotate;    /* Angstrom, degrees                 */
} mcgpu_box_desc;

/* A host-drawn trial move (the seven draws of SimCalcs::intermolecularMove,
 * SimulationStep.cpp:527-535, in their draw order). */
typedef struct {
  int32_t vertex, pad0;
  double dx, dy, dz;
  double rx, ry, rz;   /* degrees */
} mcgpu_move;

/* Per-chain counters of a device-resident run. */
typedef struct {
  double energy;          /* running total: initial system energy + sum dE */
  int64_t steps;          /* steps taken so far                            */
  int64_t accepted;       /* accepted moves so far                         */
  int64_t pairs;          /* atom pairs evaluated (old + new), if counted  */
  int32_t error;          /* device error status word: 0 none; 4 a
                             cluster-wide wait of a windowed run ran out
                             (the launch ended early); other values are
                             reserved                                       */
  int32_t ties;           /* decisions re-taken with FP64 pairs because the
                             FP32 dE fell within its rounding bound of the
                             acceptance threshold                           */
  double box[3];          /* current box edges (they change under NPT)     */
  int32_t vol_tried;      /* volume moves attempted                        */
  int32_t vol_accepted;   /* volume moves accepted                         */
  int32_t nl_builds;      /* Verlet-list builds                            */
  int32_t nl_full_scans;  /* steps screened over all molecules while a list
                             was on (trial beyond skin/2, or list stale)   */
  int32_t window_redo;    /* steps of a window (mcgpu_chain_set_window,
                             mcgpu_batch_set_window) evaluated again after
                             an earlier accepted step of the window moved
                             their molecule or one within range of it      */
  int32_t pad0;
} mcgpu_chain_stats;

/* One volume move of an NPT chain (for replay checks). */
typedef struct {
  int64_t step;           /* chain step count when the move was made       */
  int32_t accepted;
  int32_t evaluated;      /* 0 if rejected outright (the new edge would be
                             at most four times the largest molecule
                             radius)                                        */
  double e_old, e_new;    /* FP64 system energies at V and V'              */
  double dlnv, u;         /* the ln V step and the acceptance uniform      */
  double edge;            /* box edge x after the decision                 */
  int32_t fp64;           /* 0: FP32 energies (mixed) or FP64 (FP64 form);
                             1: both re-taken (double-float, then FP64);
                             2: e_new re-taken in double-float, e_old the
                             running energy                                 */
  int32_t pad0;
} mcgpu_vol_trace;

/* One step of a recorded device trajectory (for replay checks). */
typedef struct {
  int32_t mol, accepted;
  double e_old, e_new, de, u;
  int32_t fp64;           /* 1 if this step's energies are the FP64 re-take */
  int32_t pad0;
} mcgpu_trace;

typedef struct mcgpu_ctx mcgpu_ctx;
typedef struct mcgpu_box mcgpu_box;
typedef struct mcgpu_batch mcgpu_batch;
typedef struct mcgpu_server mcgpu_server;

/* ---- context ------------------------------------------------------------ */

/* Creates a context on CUDA device `device` (one GPU per context). */
int mcgpu_ctx_create(mcgpu_ctx** out, int device);
/* Destroys the context; destroy its boxes, batches and servers first. */
int mcgpu_ctx_destroy(mcgpu_ctx* ctx);
/* Makes the context launch on the caller's CUDA stream (a cudaStream_t
 * passed as a plain pointer; NULL restores the context's own stream).  The
 * caller keeps the stream alive while the context uses it. */
int mcgpu_ctx_set_stream(mcgpu_ctx* ctx, void* stream);
/* Copies the last error message of the context (or of the process when ctx
 * is NULL) into buf, NUL-terminated. */
int mcgpu_last_error(const mcgpu_ctx* ctx, char* buf, size_t len);
/* Library version string, e.g. "mcgpu_gb300 0.1 sm_103a". */
const char* mcgpu_version(void);

/* ---- plain single-chain path: the SimulationStep contract --------------- */

/* Replaces GPUCopy::copyIn (GPUCopy.cpp:97-188): uploads the box to a
 * device-resident structure of arrays.  The box keeps its own copy. */
int mcgpu_box_upload(mcgpu_ctx* ctx, const mcgpu_box_desc* desc, int precision,
                     mcgpu_box** out);
int mcgpu_box_destroy(mcgpu_box* box);
/* Replaces GPUCopy::copyOut (GPUCopy.cpp:190-222): current coordinates and
 * box edges (size may be NULL). */
int mcgpu_box_download(mcgpu_box* box, double* x, double* y, double* z,
                       double* size);

/* Replaces BruteForceCalcs::calcMolecularEnergyContribution
 * (BruteForceStep.cpp:15-46): energy of molecule curr_mol with every
 * molecule in [start_mol, n_mol) other than itself whose primary indexes
 * come within the cutoff. */
int mcgpu_mol_energy(mcgpu_box* box, int curr_mol, int start_mol, double* out);

/* Replaces SimulationStep::changeMolecule -> SimCalcs::intermolecularMove
 * (SimulationStep.cpp:520-566) with the draws supplied by the caller: saves
 * the rollback copy, rotates about the vertex atom, translates, wraps. */
int mcgpu_change_molecule(mcgpu_box* box, int mol, const mcgpu_move* mv);

/* Replaces SimulationStep::rollback -> SimCalcs::rollback
 * (SimulationStep.cpp:731-749). */
int mcgpu_rollback(mcgpu_box* box, int mol);

/* Replaces SimulationStep::calcSystemEnergy (SimulationStep.cpp:40-71) with
 * subLJ = subCharge = 0: every in-range molecule pair counted once. */
int mcgpu_system_energy(mcgpu_box* box, double* out);

/* One whole trial move in one launch: old energy, move, new energy (the
 * calls Simulation.cpp:244-250 makes), both energies returned. */
int mcgpu_move_energies(mcgpu_box* box, int mol, const mcgpu_move* mv,
                        double* e_old, double* e_new);

/* Result of mcgpu_run_plain. */
typedef struct {
  double energy0;         /* system energy at the start (calcSystemEnergy)   */
  double energy;          /* running total at the end: energy0 + sum of dE   */
  int64_t accepted, rejected;
  int64_t pairs;          /* atom pairs evaluated (old + new), counted on the
                             device                                          */
} mcgpu_plain_stats;

/* Simulation::run's NVT loop (Simulation.cpp:219-264) in C++ over the
 * contract calls above: srand(seed), then per step chooseMolecule, the
 * seven intermolecularMove draws and acceptMove's uniform from the C
 * library's rand() in the reference's order (SimulationStep.cpp:25-27,
 * 527-535, 794-803), calcMoleculeEnergy before and after changeMolecule,
 * rollback on rejection -- the calls a GpuBruteForceStep makes under the
 * reference's own loop.  fused != 0 takes the old energy, the move and the
 * new energy in one mcgpu_move_energies launch (the same draws and
 * decisions; rigid molecules only).  With intramolecular moves on
 * (mcgpu_box_set_intra) every step also makes the intramolecular move with
 * its draws, sets the step counter the width tuning reads to the loop's step
 * (starting from the topology's step_num) and the calls are made one by
 * one whatever fused says. */
int mcgpu_run_plain(mcgpu_box* box, unsigned int seed, int n_steps, int fused,
                    mcgpu_plain_stats* out);

/* The same loop run on the device: one CTA of the GPU takes every step
 * (chooseMolecule, the rigid move and, with intramolecular moves on, the
 * stages, their MC tests and the width tuning; energies; acceptMove;
 * rollback) with no host round trip.  Its draws come from the C library's
 * generator restated on the device and seeded as srand(seed) seeds it
 * (glibc's random(): the degree-31 additive feedback generator), so it draws
 * the numbers the reference's randomReal draws and takes the same decisions
 * (up to near-ties of FP64 energies summed in another order); rotations use
 * the device's sin/cos, so coordinates equal the reference's to a few ulps
 * rather than bit for bit.  The host C library's own rand() state is not
 * advanced. */
int mcgpu_run_plain_device(mcgpu_box* box, unsigned int seed, int n_steps,
                           mcgpu_plain_stats* out);
/* The device loop of n_boxes boxes of one context and one pair precision at
 * once, one CTA each, box i seeded with seeds[i]; out[i] its result (the
 * same as running it alone). */
int mcgpu_boxes_run_plain_device(mcgpu_box* const* boxes, int n_boxes,
                                 const unsigned int* seeds, int n_steps,
                                 mcgpu_plain_stats* out);

/* The first n values the restated generator gives after srand(seed)
 * (host only; for checking it against the C library). */
int mcgpu_rand_stream(unsigned int seed, int n, int32_t* out);

/* ---- flexible molecules: bonds, angles, intramolecular moves ------------ *
 *
 * The reference compiles bond stretches, angle expansions and the
 * intramolecular energy but calls them only when ENABLE_INTRA is true
 * (SimulationStep.h:15; false in its sources).  A box given a topology
 * carries the bond / angle rows; mcgpu_box_set_intra(box, 1) is ENABLE_INTRA:
 * mcgpu_mol_energy and mcgpu_system_energy then add the intramolecular
 * energy (SimulationStep.cpp:15-18), mcgpu_change_molecule follows the rigid
 * move with the intramolecular move drawing from the C library's rand()
 * (:424-428, :568-675) and mcgpu_rollback also restores the bond lengths
 * and angle sizes (:745-748).  Off by default, as in the reference.  The
 * device-resident chain forms move rigid molecules only: mcgpu_chain_run
 * refuses a box with intramolecular moves on. */

/* The bond / angle rows of SimBox (SimBox.h:160-305) as SimBoxBuilder fills
 * them (SimBoxBuilder.cpp:136-278).  Atom indexes are box atom indexes; a
 * bond's atoms and an angle's ends lie in their molecule, an angle's middle
 * may be any atom (the reference's loader gives z-matrix angles the first
 * atom of their copy set).  pair_code holds, per molecule type t (mol_type),
 * a type_natom[t] x type_natom[t] row-major matrix, the matrices
 * concatenated: 0 excluded, 1 fudge 0.5, 2 full (the exclusion and fudge
 * lists, SimBox.h:298-305).  Angle sizes are in degrees. */
typedef struct {
  int32_t n_bond, n_angle, n_type, max_intra_moves;
  const int32_t *bond_a1, *bond_a2, *bond_var;      /* bondData A1/A2/VARIABLE */
  const double *bond_k, *bond_eq, *bond_len;        /* KBOND, EQDIST, bondLengths */
  const int32_t *angle_a1, *angle_a2, *angle_mid, *angle_var;
  const double *angle_k, *angle_eq, *angle_size;    /* KANGLE, EQANGLE, angleSizes */
  const int32_t *mol_bond_start, *mol_bond_count;   /* moleculeData MOL_BOND_* */
  const int32_t *mol_angle_start, *mol_angle_count; /* moleculeData MOL_ANGLE_* */
  const int32_t *mol_type;                          /* moleculeData MOL_TYPE */
  const int32_t *type_natom;
  const uint8_t *pair_code;
  double max_bond_delta, max_angle_delta;           /* maxBondDelta, maxAngleDelta */
  int64_t step_num;                                 /* stepNum */
} mcgpu_topology_desc;

/* Tuned widths, step counter and the tuning counters of a box
 * (maxBondDelta, maxAngleDelta, stepNum, numBondMoves, numAcceptedBondMoves,
 * numAngleMoves, numAcceptedAngleMoves; SimBox.h:23-72). */
typedef struct {
  double max_bond_delta, max_angle_delta;
  int64_t step_num;
  int64_t bond_moves, bond_accepted, angle_moves, angle_accepted;
} mcgpu_intra_state;

/* Uploads the topology (replaces any earlier one; the counters start at 0).
 * Checks every index against the box; a bond or angle end outside its
 * molecule is MCGPU_ERR_INVALID (the reference would index its union-find
 * scratch out of range). */
int mcgpu_box_set_topology(mcgpu_box* box, const mcgpu_topology_desc* topo);
/* ENABLE_INTRA for this box (needs a topology). */
int mcgpu_box_set_intra(mcgpu_box* box, int enable);
/* SimCalcs::calcIntraMolecularEnergy (SimulationStep.cpp:80-129): angle and
 * bond terms of the variable entries when the box has variable angles /
 * bonds, and when it has either the LJ and Coulomb terms of every
 * non-excluded atom pair of the molecule (fudge pairs halved, no cutoff). */
int mcgpu_intra_energy(mcgpu_box* box, int mol, double* out);
/* SimCalcs::stretchBond (:257-315): bond index within the molecule. */
int mcgpu_stretch_bond(mcgpu_box* box, int mol, int bond, double dist);
/* SimCalcs::expandAngle (:148-239): angle index within the molecule,
 * degrees. */
int mcgpu_expand_angle(mcgpu_box* box, int mol, int angle, double deg);
/* SimCalcs::saveBonds / saveAngles (:678-701). */
int mcgpu_save_intra(mcgpu_box* box, int mol);
/* SimCalcs::intramolecularMove (:568-675), its draws from the C library's
 * rand(): save, stretch a random set of bonds, count the MC test, the same
 * for the angles, tune the widths when the step counter is a nonzero
 * multiple of 1000. */
int mcgpu_intramolecular_move(mcgpu_box* box, int mol);
/* Sets stepNum, the counter the width tuning reads (Simulation::run
 * increments the reference's after every step, Simulation.cpp:263). */
int mcgpu_intra_set_step(mcgpu_box* box, int64_t step);
/* Current bond lengths [n_bond], angle sizes [n_angle] (either may be NULL)
 * and state. */
int mcgpu_intra_get(mcgpu_box* box, double* bond_len, double* angle_size,
                    mcgpu_intra_state* state);

/* ---- device-resident chain (Philox RNG, on-device accept) --------------- */

/* Runs n_steps Metropolis steps of this box as chain `chain_id` with the
 * Philox4x32-10 key `seed`, proposals drawn on the device; the running
 * energy starts from a full system energy on the first call.  If trace is
 * non-NULL it receives n_steps records. */
int mcgpu_chain_run(mcgpu_box* box, uint64_t seed, uint32_t chain_id,
                    int n_steps, int rotation, mcgpu_chain_stats* stats,
                    mcgpu_trace* trace);
/* Steps per window of this box's device-resident runs: k = 1 (one step at a
 * time, the default), 2, 4, 8 or 16 (16: a non-portable cluster size).  With k > 1 a chain is advanced by a
 * thread-block cluster of k CTAs: each window's k moves (known in advance:
 * counter-based draws) are evaluated at once, one per CTA, against the state
 * at the window's start; then every CTA takes the k decisions in step order
 * and evaluates a step again on the current state when an earlier accepted
 * step of the window moved its molecule or a molecule within range of it.
 * Decisions, coordinates and counters equal those of k = 1; only the FP32
 * summation order of re-evaluated steps can differ.  Needs k CTAs on k SMs
 * of one GPC (refused with MCGPU_ERR_UNSUPPORTED where none fits). */
int mcgpu_chain_set_window(mcgpu_box* box, int k);

/* ---- batched chains: one persistent kernel advances many chains --------- */

/* Uploads n_chains independent boxes (uneven sizes and temperatures allowed)
 * into one device pool; chain c uses Philox key seeds[c] and counter
 * chain id c.  precision is MCGPU_PREC_MIXED in this build.  The running
 * energies start from FP32-pair system energies (double-float sums; their
 * error bound is carried with the chain); mcgpu_batch_system_energy gives
 * FP64 totals. */
int mcgpu_batch_create(mcgpu_ctx* ctx, int n_chains, const mcgpu_box_desc* descs,
                       const uint64_t* seeds, int rotation, mcgpu_batch** out);
int mcgpu_batch_destroy(mcgpu_batch* batch);
/* Advances every chain by n_steps steps (launches of steps_per_launch steps,
 * replayed from a captured CUDA graph).  Asynchronous on the batch stream
 * unless sync != 0. */
int mcgpu_batch_run(mcgpu_batch* batch, int n_steps, int sync);
/* Chooses threads per CTA, chains per CTA, lanes per neighbour molecule and
 * steps per launch by timing candidate tiles on this batch, trial_steps
 * steps each, every timed launch starting from a cleared L2 (the rows are
 * saved first and restored after every trial and at the end, so the batch
 * continues from where it was).  Allocates a scratch buffer of twice the L2
 * size for the duration of the call. */
int mcgpu_batch_autotune(mcgpu_batch* batch, int trial_steps);
/* Sets the tile explicitly: threads per CTA (32..512, a multiple of 32),
 * chains per CTA (dividing its warps), steps per launch (>= 1), and lanes
 * per neighbour molecule (a power of two <= 32 capping every chain's
 * default; 0 keeps the defaults: one lane for a chain of one species of at
 * most 4 atoms, else the power of two at or above its largest molecule).
 * Results do not depend on the first three; the lanes change the FP32
 * summation order and so the last bits of the energies. */
int mcgpu_batch_set_tile(mcgpu_batch* batch, int threads, int chains_per_cta,
                         int steps_per_launch, int lanes_per_molecule);
int mcgpu_batch_get_tile(mcgpu_batch* batch, int* threads, int* chains_per_cta,
                         int* steps_per_launch, int* lanes_per_molecule);
/* Windows of k steps (1, 2, 4, 8, 16) for the batch's chains, as
 * mcgpu_chain_set_window: one cluster of k CTAs per chain, each CTA one
 * group of the tile's threads (the tile must have one chain per CTA and at
 * least k warps).  For a few large chains; a batch of many chains already
 * fills the device one chain per group. */
int mcgpu_batch_set_window(mcgpu_batch* batch, int k);
/* Like mcgpu_batch_run (synchronous, no graph) and records every step:
 * out[c * n_steps + s] is step s of chain c.  If vol_out is non-NULL it
 * receives the volume moves of an NPT batch: vol_out[c * (n_steps /
 * interval + 1) + k] is the k-th volume move of chain c in this call. */
int mcgpu_batch_run_traced(mcgpu_batch* batch, int n_steps, mcgpu_trace* out,
                           mcgpu_vol_trace* vol_out);
/* Makes the batch isobaric (NPT): after every `interval` steps of a chain
 * (its step count a multiple of interval) it attempts one volume move,
 * ln V' = ln V + U(-max_dlnv[c], max_dlnv[c]) with every edge scaled by
 * exp(dlnv / 3) and the molecules' centres (first primary atoms) scaled
 * with it, accepted by the isobaric criterion
 *   exp(-(U(V') - U(V) + P (V' - V)) / kT + (N + 1) dlnv) >= u
 * at pressure_atm[c] atmospheres (1 atm = 1.4584e-5 kcal/mol/A^3), with
 * U(V) and U(V') full FP64 system energies; the chain's running energy then
 * restarts from the FP64 energy of the volume it keeps.  The reference's
 * NPTEnsemble (Ensemble.cpp:9-23, SimulationStep.cpp:476-518) is the
 * counterpart; its fixed factor 1.1 and unitless P dV are not reproduced.
 * interval 0 makes the batch NVT again.  max_dlnv in (0, 0.1].
 * precision MCGPU_PREC_FP64 computes U(V), U(V') with FP64 pair terms;
 * MCGPU_PREC_MIXED with FP32 pair terms summed in double-float, re-taking
 * in FP64 only the moves whose criterion argument lies within the FP32
 * rounding bound of ln u (so the decisions are the FP64 ones; the kept
 * energy carries the FP32-pair error).  GB300 issues FP64 at 1/64 of the
 * FP32 rate, which makes the FP64 form the dominant cost of frequent volume
 * moves on large boxes. */
int mcgpu_batch_set_npt(mcgpu_batch* batch, int interval, const double* pressure_atm,
                        const double* max_dlnv, int precision);
/* Verlet neighbour lists with the given skin (Angstrom; <= 0 turns them
 * off) for every chain of a batch, or for the device-resident chain of a
 * box.  Built on the GPU from a cell list on the molecules' anchors (cells
 * at least rc + skin + 2 * primary radius wide), rebuilt between launches
 * once a molecule has moved more than skin/2 since the last build; while a
 * trial placement is farther than that the step screens all molecules.
 * The in-range sets, and so the trajectories, are those of the full scan.
 * Replaces the reference's VerletStep / NLCStep strategies
 * (VerletStep.cpp:119-207, NLCStep.cpp:125-243) for the chain forms. */
int mcgpu_batch_set_verlet(mcgpu_batch* batch, double skin);
/* Long-range LJ correction in the isobaric criterion: lrc_v[c] = E_LRC * V
 * of chain c (kcal/mol * A^3; the correction scales as 1/V at fixed N), so a
 * volume move adds lrc_v (1/V' - 1/V) to dU.  0 (the default) leaves it out.
 * The reference computes E_LRC once at the start (SerialCalcs.cpp:37-107,
 * Simulation.cpp:81) and never on a volume change.  Running energies stay
 * pair energies; E_LRC at the current box is lrc_v / V. */
int mcgpu_batch_set_lrc(mcgpu_batch* batch, const double* lrc_v);
int mcgpu_box_set_verlet(mcgpu_box* box, double skin);
/* Pair arithmetic of a batch's steps.  MCGPU_PREC_MIXED (the default): FP32
 * pair terms, double-float sums, the FP64 pairs only for the decisions that
 * fall within the FP32 rounding bound of the threshold.  MCGPU_PREC_FP64:
 * every step with the reference's FP64 pair arithmetic (BruteForceStep.cpp:
 * 48-79, SimulationStep.cpp:317-385) on the chain state's FP64 positions.
 * The decisions, and so the trajectories, are the same in both; the running
 * energy of the FP64 form carries FP64 rounding only.  GB300 issues FP64 at
 * 1/64 of the FP32 rate, so the FP64 form is the slower one.  The stats'
 * `ties` then count every step. */
int mcgpu_batch_set_precision(mcgpu_batch* batch, int precision);
int mcgpu_batch_sync(mcgpu_batch* batch);
int mcgpu_batch_stats(mcgpu_batch* batch, mcgpu_chain_stats* stats);
/* Coordinates of chain c (arrays sized like its descriptor). */
int mcgpu_batch_download(mcgpu_batch* batch, int chain, double* x, double* y,
                         double* z);
/* Coordinates of every chain, concatenated in chain order (arrays of the
 * batch's total atom count): three copies for the whole batch. */
int mcgpu_batch_download_all(mcgpu_batch* batch, double* x, double* y, double* z);
/* Checkpoint of a batch: the resumable device state (coordinates, anchors,
 * orientations, screen positions, every chain header with its running
 * energy, counters and Philox step counter, the Verlet lists, the NPT
 * phase) as an opaque host blob.  With buf == NULL only *used is set (the
 * size).  The reference's resumable state is the text .state file
 * (StateScanner::outputState, StateScanner.cpp:545-597, read back by
 * loadBoxData, FileUtilities.cpp:119-163), which keeps six significant
 * digits and restarts the RNG from the seed; this blob resumes bit for bit. */
int mcgpu_batch_checkpoint(mcgpu_batch* batch, void* buf, size_t cap, size_t* used);
/* Restores a checkpoint into a batch created from the same boxes, with the
 * same Verlet skin and NPT interval set; the batch then continues exactly
 * as the checkpointed one would have.  MCGPU_ERR_INVALID for a blob of
 * another layout or settings (nothing is changed then). */
int mcgpu_batch_restore(mcgpu_batch* batch, const void* buf, size_t len);
/* Recomputes every chain's total energy from scratch (FP64 accumulate) into
 * out[n_chains]; the running totals are not changed. */
int mcgpu_batch_system_energy(mcgpu_batch* batch, double* out);

/* ---- serving: continuous batching of simulation jobs ------------------- */

/* A server keeps many jobs (independent chains) resident on one GPU and
 * advances them together in rounds of round_steps steps of the persistent
 * chain kernel.  Jobs arriving while others run wait in a FIFO queue and are
 * admitted between rounds as slots and memory free up (a later, smaller job
 * may pass a larger one that does not fit yet); a job leaves the pool at the
 * end of the round in which it reaches its step count.  A job's results
 * depend only on its own description (box, seed, chain id, steps, ensemble)
 * and the server's tile: the same alone as in any mix. */
typedef struct {
  uint64_t hbm_budget_bytes;  /* admission limit on resident job state       */
  int64_t max_atoms;          /* arena capacity in atoms (0: from the budget,
                                 at 4 atoms per molecule)                    */
  int64_t max_molecules;      /* arena capacity in molecules (0: as above)   */
  int32_t max_slots;          /* jobs resident at once (1..4096)             */
  int32_t round_steps;        /* steps per round; NPT jobs make a volume move
                                 every round_steps steps                     */
  int32_t max_mol_atoms;      /* largest molecule a job may hold (<= 64)     */
  int32_t rotation;           /* MCGPU_ROT_EULER or MCGPU_ROT_AXIS          */
  int32_t threads, chains_per_cta, lanes_per_molecule; /* chain-kernel tile,
                                 fixed for the server's life (0: defaults)   */
  int32_t pad0;
} mcgpu_server_config;

typedef struct {
  const mcgpu_box_desc* box;  /* copied at submit                          */
  uint64_t seed;              /* Philox key                                */
  uint32_t chain_id;          /* Philox counter id                         */
  int32_t npt;                /* 1: isobaric volume moves                  */
  int32_t vol_precision;      /* NPT energies: MCGPU_PREC_FP64 or _MIXED (see
                                 mcgpu_batch_set_npt)                      */
  int32_t pad1;
  int64_t n_steps;            /* trial moves to run                        */
  double pressure_atm;        /* NPT pressure                              */
  double max_dlnv;            /* NPT ln V step bound, (0, 0.1]             */
  double *x_out, *y_out, *z_out; /* final coordinates (n_atom each), may be
                                 NULL; must stay valid until the job's result
                                 is taken by mcgpu_server_results          */
  double lrc_v;               /* NPT: E_LRC * V of the job's long-range LJ
                                 correction in the volume criterion (see
                                 mcgpu_batch_set_lrc); 0 for none           */
} mcgpu_job_desc;

typedef struct {
  int64_t job_id;
  double energy;              /* running total at the end                  */
  int64_t steps, accepted;
  int32_t vol_tried, vol_accepted;
  double box[3];
  double t_submit, t_admit, t_done; /* seconds on the server's clock        */
  int64_t footprint_bytes;    /* device bytes the job held                 */
  int32_t error, ties;
} mcgpu_job_result;

int mcgpu_server_create(mcgpu_ctx* ctx, const mcgpu_server_config* cfg,
                        mcgpu_server** out);
int mcgpu_server_destroy(mcgpu_server* srv);
/* Queues a job (its rows are copied).  MCGPU_ERR_CAPACITY if the job could
 * never be admitted (larger than the budget, the arena or the molecule
 * limit). */
int mcgpu_server_submit(mcgpu_server* srv, const mcgpu_job_desc* job, int64_t* job_id);
/* One round: admits what fits (uploads overlap the round in flight), waits
 * for the round in flight, retires the jobs it finished (coordinates to
 * x_out/y_out/z_out), admits again and launches the next round
 * (asynchronously).  Returns without work when nothing is queued or running. */
int mcgpu_server_step(mcgpu_server* srv);
/* Steps until every submitted job has finished. */
int mcgpu_server_drain(mcgpu_server* srv);
int mcgpu_server_status(mcgpu_server* srv, int* running, int* queued, int64_t* finished,
                        uint64_t* bytes_in_use);
/* Moves up to max finished jobs' results to out (oldest first); *n gets the
 * count. */
int mcgpu_server_results(mcgpu_server* srv, mcgpu_job_result* out, int max, int* n);
/* Seconds on the server's clock (the clock of t_submit/t_admit/t_done). */
double mcgpu_server_clock(const mcgpu_server* srv);
/* Work counters of the server, for throughput and roofline figures (no
 * reference counterpart): *pairs the atom pairs (old + new placement) that
 * the retired jobs evaluated, counted on the device; *gpu_seconds the GPU
 * time of the rounds completed so far (chain kernel and volume phase,
 * between CUDA events on the compute stream); *rounds their number.  Any
 * pointer may be NULL. */
int mcgpu_server_counters(mcgpu_server* srv, int64_t* pairs, double* gpu_seconds,
                          int64_t* rounds);

/* ---- no-allocation system energy ---------------------------------------- */

/* No counterpart in the reference: an extra entry point for callers that may
 * not allocate device memory through this library -- an OpenACC/OpenMP
 * offload program whose SimBox rows already live in its own device data
 * region, or an application whose device memory belongs to another
 * allocator (a caching allocator, a fixed arena) that forbids allocations by
 * third-party code.  It computes what mcgpu_system_energy computes with FP64
 * pairs (SimulationStep::calcSystemEnergy, SimulationStep.cpp:40-71, with
 * subLJ = subCharge = 0) without any context, box or allocation:
 *   rows   -- a descriptor whose row pointers are DEVICE pointers of the
 *             current CUDA device (only n_*, the rows, size and cutoff are
 *             read);
 *   out    -- a DEVICE pointer to one double, written by the call;
 *   stream -- a cudaStream_t as a plain pointer (NULL = default stream).
 * The call is asynchronous: *out is ready when the stream reaches it.
 * Its per-molecule partials go to a fixed array in device memory that the
 * library reserves on every GPU it is loaded on (256 KiB), so n_mol is at
 * most 32768; larger boxes return MCGPU_ERR_UNSUPPORTED.  Nothing has to be
 * zeroed first: every partial a call reads, it has written.  Calls share the
 * array, so two calls that can run at the same time on one device (two
 * streams without ordering, two host threads) race and give wrong sums.  The
 * first call on each device looks up the array's address with that device
 * current; make that first call before any stream capture.  The address is
 * cached per device together with the id of the context it was found in: a
 * call made after the application reset the device or re-created its
 * primary context looks it up again (that call is then a first call too).
 * Rows that index out of range give NaN instead of being read; a molecule
 * with no primary indexes contributes nothing, as in moleculesInRange.  A
 * CUDA error the caller left pending is neither cleared nor reported as
 * this call's.  Errors: MCGPU_ERR_INVALID, MCGPU_ERR_UNSUPPORTED,
 * MCGPU_ERR_CUDA; text via mcgpu_last_error(NULL). */
int mcgpu_system_energy_static(const mcgpu_box_desc* rows, double* out, void* stream);

/* ---- initial configuration (host only, no GPU) -------------------------- */

/* Places n points uniformly in [0, L)^3 with minimum-image separation >= dmin
 * by random sequential addition (every rejected candidate redrawn), seeded;
 * out[3*i + d].  The reference builds its initial boxes on the host as an
 * FCC lattice (FileUtilities.cpp:550-642); this is the random-start builder
 * of the synthetic workloads.  Returns 0, 1 (bad argument) or 2 (no room). */
int mcgpu_build_centres(int n, double L, double dmin, uint64_t seed, double* out);

#ifdef __cplusplus
}
#endif
#endif
