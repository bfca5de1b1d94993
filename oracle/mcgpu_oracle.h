/*
 * mcgpu_oracle.h -- CPU FP64 restatement of MCGPU's Metropolis trial-move
 * energy path.  TEST INFRASTRUCTURE ONLY: this is the checker the CUDA path is
 * compared against (and the timed CPU baseline); nothing in the product links
 * or calls it.
 *
 * Every function restates one reference function (file:line in each comment)
 * with the same arithmetic and the same summation order, so that on the same
 * inputs it returns the same bits as the reference compiled with `g++ -O3`
 * (checked against the compiled reference by tests/test_oracle_pins.py and
 * against committed golden vectors by tests/test_oracle_golden.py).
 */
#ifndef MCGPU_ORACLE_H
#define MCGPU_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Structure-of-arrays box, one row per SimBox row (src/Metropolis/SimBox.h:120-149). */
typedef struct {
  int n_mol, n_atom, n_pidx, largest_mol;
  double *x, *y, *z;                  /* atomCoordinates[X/Y/Z][n_atom]        */
  double *sigma, *epsilon, *charge;   /* atomData[ATOM_SIGMA/EPSILON/CHARGE]    */
  int *mol_start, *mol_len;           /* moleculeData[MOL_START/MOL_LEN]        */
  int *mol_pidx_start, *mol_pidx_count; /* moleculeData[MOL_PIDX_START/COUNT]   */
  int *pidx;                          /* primaryIndexes[n_pidx] (absolute)      */
  double *rb_x, *rb_y, *rb_z;         /* rollBackCoordinates[3][largest_mol]    */
  double size[3];
  double cutoff, kT, max_translate, max_rotate;
} orc_box;

/* One trial move.  mode 0: Euler X->Y->Z in degrees about the vertex atom
 * (the reference form); mode 1: rotation by r3 degrees about the unit axis
 * (r0, r1, r2) through the vertex atom (the random-axis form). */
typedef struct {
  int mol, vertex, mode, pad;
  double dx, dy, dz;
  double r0, r1, r2, r3;
  double u;          /* acceptance uniform (used only when dE >= 0) */
} orc_move;

typedef struct {
  int mol, accepted;
  double e_old, e_new, de, u;
} orc_trace;

double orc_make_periodic(double x, double dim_len);
double orc_atom_dist2(const orc_box* b, int a1, int a2);
double orc_blend(double a, double c);
double orc_lj(const orc_box* b, int a1, int a2, double r2);
double orc_charge(const orc_box* b, int a1, int a2, double r);
int orc_molecules_in_range(const orc_box* b, int p1s, int p1e, int p2s, int p2e);
double orc_mol_pair_energy(const orc_box* b, int m1, int m2);
double orc_mol_energy(const orc_box* b, int curr, int start);
double orc_system_energy(const orc_box* b);
double orc_mol_energy_abs(const orc_box* b, int curr, int start);
double orc_mol_energy_absk(const orc_box* b, int curr, int start);
int orc_count_pairs(const orc_box* b, int curr, long long* mol_pairs, long long* atom_pairs);

void orc_keep_in_box(orc_box* b, int mol);
void orc_wrap_all(orc_box* b);
void orc_apply_move(orc_box* b, const orc_move* mv);
void orc_rollback(orc_box* b, int mol);
int orc_accept(double de, double kT, double u);
double orc_random_real(double start, double end, int r);

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
void orc_philox_move(uint64_t seed, uint32_t chain, uint64_t step, int n_mol,
                     const int* mol_len, double max_t, double max_r, int mode,
                     orc_move* mv);
double orc_chain_run(orc_box* b, uint64_t seed, uint32_t chain, uint64_t step0,
                     int n_steps, int mode, double e0, orc_trace* trace,
                     long long* n_accepted);
double orc_chains_run_mt(orc_box* boxes, int n_chains, const uint64_t* seeds,
                         uint64_t step0, int n_steps, int mode, int n_threads,
                         long long* total_moves);

void orc_resize_box_centres(orc_box* b, double scale);
int orc_accept_volume(double de, double p_kcal_per_a3, double v_old, double v_new,
                      int n_mol, double kT, double u);

#ifdef __cplusplus
}
#endif
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- device-resident chain form (FP32 moves on a fixed-point + FP32
 * offset state), mirrored from its definition so the CPU state equals the
 * device state bit for bit; energies are the reference's FP64 arithmetic on
 * the FP64 rows x = anchor * L / 2^32 + offset. */
typedef struct {
  orc_box* b;          /* FP64 rows, kept equal to the state            */
  uint32_t* A;         /* [3 * n_mol] anchors, fixed point of the edge  */
  float* q;            /* [4 * n_mol] unit quaternions (w, x, y, z)     */
  float* tpl;          /* [3 * n_atom] template offsets                 */
  float* off;          /* [3 * n_atom] current offsets                  */
  int rot_mode;
} orc_chain;

typedef struct {
  int mol, vertex;
  float dx, dy, dz;
  float qw, qx, qy, qz;
  float u;
} orc_movef;

void orc_fchain_init(orc_chain* c);
void orc_fchain_draw(const orc_chain* c, uint64_t seed, uint32_t chain, uint64_t step,
                    orc_movef* mv);
double orc_fchain_run(orc_chain* c, uint64_t seed, uint32_t chain, uint64_t step0,
                     int n_steps, double e0, orc_trace* trace, long long* n_accepted);
/* The same loop in windows of K steps, each step evaluated first on the
 * state at its window's start and again only when an earlier accepted step
 * of the window moved its molecule or one in range of it; *n_redo counts
 * those.  Returns what orc_fchain_run returns, with the same trace.
 * in_range_rule = 0 plants a mistake (only same-molecule steps are evaluated
 * again), for tests. */
double orc_fchain_run_window(orc_chain* c, uint64_t seed, uint32_t chain, uint64_t step0,
                             int n_steps, int K, double e0, orc_trace* trace,
                             long long* n_accepted, long long* n_redo, int in_range_rule);
void orc_sincos_f32(float x, float* s, float* c);
int orc_fchain_volume(orc_chain* c, uint64_t seed, uint32_t chain, uint64_t step,
                      double p_kcal, double max_dlnv, float rad_max, double lrc_v, double* energy,
                      double* e_old, double* e_new, double* dlnv_out, double* u_out);

/* Synthetic input generation: molecule centres by random sequential
 * addition (the same points as the product's input builder). */
int orc_build_centres(int n, double L, double dmin, uint64_t seed, double* out);

/* ---- flexible molecules: the bond / angle rows of the SimBox
 * (src/Metropolis/SimBox.h:160-305) and the reference's intramolecular
 * functions as they run with ENABLE_INTRA true. */
typedef struct {
  int n_bond, n_angle, n_type, max_intra_moves;
  int *bond_a1, *bond_a2, *bond_var;          /* bondData[A1/A2/VARIABLE]       */
  double *bond_k, *bond_eq, *bond_len;        /* bondData[KBOND/EQDIST], bondLengths */
  double* bond_len_rb;                        /* rollBackBondLengths            */
  int *angle_a1, *angle_a2, *angle_mid, *angle_var;
  double *angle_k, *angle_eq, *angle_size;    /* angleData[KANGLE/EQANGLE], angleSizes */
  double* angle_size_rb;                      /* rollBackAngleSizes             */
  int *mol_bond_start, *mol_bond_count, *mol_angle_start, *mol_angle_count, *mol_type;
  int *type_natom, *type_off;                 /* per type: atoms, offset in pair_code */
  unsigned char* pair_code;                   /* 0 excluded, 1 x0.5, 2 full     */
  int* uf;                                    /* union-find scratch [largest_mol] */
  double max_bond_delta, max_angle_delta;
  long long step_num;
  long long bond_moves, bond_accepted, angle_moves, angle_accepted;
  int flex_bonds, flex_angles;
} orc_topo;

double orc_bond_energy(const orc_topo* t, int mol);
double orc_angle_energy(const orc_topo* t, int mol);
double orc_intra_energy(const orc_box* b, const orc_topo* t, int mol);
void orc_stretch_bond(orc_box* b, orc_topo* t, int mol, int bond, double dist);
void orc_expand_angle(orc_box* b, orc_topo* t, int mol, int angle, double deg);
void orc_save_intra(orc_topo* t, int mol);
void orc_rollback_intra(orc_topo* t, int mol);
void orc_intramolecular_move(orc_box* b, orc_topo* t, int mol);
double orc_system_energy_intra(const orc_box* b, const orc_topo* t);
double orc_run_plain_intra(orc_box* b, orc_topo* t, int steps, double e0, int* accepted);

#ifdef __cplusplus
}
#endif
