/*
 * spss_oracle — CPU restatement (FP64, reference AoS layout) of the
 * pairwise-interaction hot path of raven91/spssLangevinIntegration.
 *
 * TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg load this library, and only as the checker or the timed
 * CPU reference; the GPU product never calls it and has no CPU fallback.
 *
 * Parity status: pinned.  tests/test_oracle_golden.py checks every routine
 * below against fixtures produced by the reference's own sources compiled
 * unmodified (oracle/Makefile target `ref`, fixtures in tests/golden/).
 *
 * Layout: state is `double[n*s]`, s = 4 (x, y, phi, omega) for the first-order
 * model and s = 6 (x, y, v_x, v_y, phi, omega) for the second-order model,
 * exactly as the reference stores it.  The box is the unit square.
 *
 * Two routines have no reference implementation and are restated here from
 * the reference's own building blocks (each says so where it is defined):
 * the second-order Verlet-list interaction and the second-order strong
 * order 1.5 stochastic Taylor stepper.
 */
#ifndef SPSS_ORACLE_H
#define SPSS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum
{
  SPO_DISPATCH = 0,          /* EvaluateRhs: the reference's rho-based choice */
  SPO_ALL_PAIRS = 1,
  SPO_LINKED_LIST = 2,
  SPO_VERLET = 3,            /* Verlet list with an O(N^2) rebuild */
  SPO_LINKED_LIST_VERLET = 4,/* Verlet list rebuilt from the cell list */
  SPO_GLOBAL_FIELD = 5       /* first order only: global polar order field */
};

typedef struct spo_params
{
  int model;      /* 1: first order, 2: second order */
  int flavor;     /* first order: 0 = ParticleSystemFirstOrder, 1 = ParticleSystemFirstOrderPtr */
  int n;          /* number of particles */
  double v0, xi, xi_r, D_r, xi_phi, D_phi, sigma, rho, alpha;
  double r_max;   /* Verlet list radius; the reference's first order uses rho + 0.05 */
  int nc_verlet;  /* cells per side for the linked-list + Verlet build; 0 = int(1/rho) */
} spo_params;

typedef struct spo_system spo_system;
typedef struct spo_stepper spo_stepper;

spo_system *spo_create(const spo_params *p);
void spo_destroy(spo_system *sys);
void spo_set_threads(int threads);
int spo_get_threads(void);

void spo_set_higher_order(spo_system *sys, int on);
void spo_set_natural_frequencies(spo_system *sys, const double *freqs);

/* EvaluateRhs / EvaluateInteractionsWith*: returns 0 or -1 on a bad variant. */
int spo_evaluate(spo_system *sys, int variant, const double *state, const double *k_prev, double *k_next,
                 double k_coef, double dt);
void spo_get_complementary_force(const spo_system *sys, double *out);

void spo_calculate_max_displacement(spo_system *sys, const double *total_displacement);
double spo_accumulated_displacement(const spo_system *sys);
int spo_should_update_lists(const spo_system *sys);
void spo_set_should_update_lists(spo_system *sys, int flag);
int spo_uses_verlet_list(const spo_system *sys);

/* Cell and Verlet lists of the most recent build (CSR). */
int spo_num_cells_per_side(const spo_system *sys, int verlet_grid);
void spo_get_pre_linked_list(const spo_system *sys, int *out);
long spo_get_cells(const spo_system *sys, int *offsets, int *members);
long spo_get_verlet(const spo_system *sys, int *offsets, int *entries);

/* Steppers.  `normals` holds the Gaussian draws of one step in the
 * reference's draw order (see each stepper); it may be NULL for RK4. */
spo_stepper *spo_stepper_create(int n, int s);
void spo_stepper_destroy(spo_stepper *st);
int spo_rk4_step(spo_system *sys, spo_stepper *st, int variant, double *state, double t, double dt);
int spo_se_step(spo_system *sys, spo_stepper *st, int variant, double *state, double t, double dt,
                const double *normals);
int spo_srk_step(spo_system *sys, spo_stepper *st, int variant, double *state, double t, double dt,
                 const double *normals);
int spo_normals_per_particle(int model, int stepper);

void spo_apply_pbc(int n, int s, double *state);
/* out = {|<e^{i phi}>|, arg, |<v/|v|>| (second order; first order: same as phase), arg} */
void spo_order_parameters(int model, int n, const double *state, double *out);

/* Counter-based Philox4x32-10 normals (Box-Muller) used by the CPU baseline
 * leg, which times the port with its own noise. */
void spo_philox_normals(unsigned long long seed, unsigned long long step, int stream, long count, double *out);

#ifdef __cplusplus
}
#endif

#endif
