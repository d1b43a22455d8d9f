/*
 * spss_oracle.c — CPU restatement of the reference hot path.  TEST
 * INFRASTRUCTURE (see spss_oracle.h): the GPU product never calls this.
 *
 * Every routine cites the reference file:line it restates.  Floating-point
 * expressions keep the reference's operation order and the library is built
 * with -ffp-contract=off, so with the same inputs it reproduces the
 * reference's FP64 results bit for bit (checked against the compiled
 * reference in tests/test_oracle_golden.py).
 *
 * Parallelism mirrors the reference's particle-index decomposition
 * (Parallelization/Thread.cpp:18-23): each particle's sums are private, so
 * the OpenMP loops give the same bits as the serial loop.
 */
#include "spss_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct
{
  int *data;
  int len, cap;
} ilist;

static void ilist_push(ilist *l, int v)
{
  if (l->len == l->cap)
  {
    l->cap = l->cap ? 2 * l->cap : 16;
    l->data = (int *) realloc(l->data, (size_t) l->cap * sizeof(int));
  }
  l->data[l->len++] = v;
}

struct spo_system
{
  spo_params p;
  int s;
  double rho_squared, cos_alpha, sin_alpha;
  double r_min;
  int nc, nc_verlet;          /* cells per side: linked list, Verlet build */
  double *rk;                 /* stage state, the reference's rk_system_state */
  double *af, *card, *caf;    /* alignment force, cardinality, complementary force */
  double *nat_freq;
  int *pll;                   /* pre_linked_list_: cell id per particle */
  int *cell_off, *cell_mem;   /* linked_list_ as CSR, members ascending */
  int cells_built;            /* number of cells in the current CSR */
  ilist *verlet;              /* verlet_list_ */
  double accumulated_displacement;
  int should_update_lists;
  int uses_verlet_list;
  int higher_order;
};

struct spo_stepper
{
  int n, s;
  double *k1, *k2, *k3, *k4, *td, *det, *stoch;
};

static int g_threads = 1;

void spo_set_threads(int threads)
{
  g_threads = threads > 0 ? threads : 1;
}

int spo_get_threads(void)
{
  return g_threads;
}

/* ------------------------------------------------------------------ PBC */

/* PeriodicBoundaryConditions::ClassAEffectiveParticleDistance
 * (BoundaryConfiguration/PeriodicBoundaryConditions.cpp:26-38), unit box. */
static inline double pbc_class_a(double d)
{
  return d - (double) (int) (d * 2.0 * 1.0) * 1.0;
}

/* PeriodicBoundaryConditions::ClassCEffectiveParticleDistanceUnsigned
 * (PeriodicBoundaryConditions.cpp:107-119), unit box. */
static inline double pbc_class_c(double d)
{
  d = fabs(d);
  return d - (double) (int) (d * 1.0 + 0.5) * 1.0;
}

/* PeriodicBoundaryConditions::ApplyPeriodicBoundaryConditions(x, y, ...)
 * (PeriodicBoundaryConditions.cpp:121-125). */
static inline double pbc_wrap(double x)
{
  return x - floor(x * 1.0) * 1.0;
}

/* The second-order classes wrap a position only when it has left the box
 * (ParticleSystemSecondOrder.cpp:323-326, :382-385). */
static inline void wrap_if_outside(double *x, double *y)
{
  if (*x < 0.0 || *x >= 1.0 || *y < 0.0 || *y >= 1.0)
  {
    *x = pbc_wrap(*x);
    *y = pbc_wrap(*y);
  }
}

/* int(x / x_size * num_subcells) (ParticleSystemFirstOrder.cpp:277-279).  A
 * wrapped coordinate can round to exactly 1.0 (or x*nc can round up to nc),
 * which the reference turns into an out-of-range cell; it is clamped here. */
static inline int cell_coord(double x, int nc)
{
  int c = (int) (x / 1.0 * nc);
  if (c >= nc) c = nc - 1;
  if (c < 0) c = 0;
  return c;
}

/* AdjustNeighboringCellToPeriodicBoundaries (ParticleSystemFirstOrder.cpp:651-668). */
static inline int adjust_cell(int c, int nc)
{
  if (c < 0) return nc - 1;
  if (c >= nc) return 0;
  return c;
}

/* neighboring_cells_ order (ParticleSystemFirstOrder.cpp:47-52). */
static const int kStencil[9][2] = {{-1, -1}, {0, -1}, {1, -1}, {-1, 0}, {0, 0}, {1, 0}, {-1, 1}, {0, 1}, {1, 1}};

void spo_apply_pbc(int n, int s, double *state)
{
  /* ApplyPeriodicBoundaryConditions(std::vector<Real>&) (PeriodicBoundaryConditions.cpp:127-135). */
  for (int i = 0; i < n; ++i)
  {
    state[(long) s * i] -= floor(state[(long) s * i] * 1.0) * 1.0;
    state[(long) s * i + 1] -= floor(state[(long) s * i + 1] * 1.0) * 1.0;
  }
}

/* ---------------------------------------------------------- construction */

spo_system *spo_create(const spo_params *p)
{
  if (!p || (p->model != 1 && p->model != 2) || p->n <= 0 || !(p->rho > 0.0)) return NULL;
  spo_system *sys = (spo_system *) calloc(1, sizeof(spo_system));
  sys->p = *p;
  sys->s = (p->model == 1) ? 4 : 6;
  sys->rho_squared = p->rho * p->rho;
  sys->cos_alpha = cos(p->alpha);
  sys->sin_alpha = sin(p->alpha);
  sys->r_min = p->rho;
  if (!(sys->p.r_max > 0.0)) sys->p.r_max = p->rho + 0.05; /* ParticleSystemFirstOrderPtr.cpp:97-98 */
  sys->nc = (int) (1.0 / p->rho);                           /* ParticleSystemFirstOrder.cpp:37-38 */
  if (sys->nc < 1) sys->nc = 1;
  sys->nc_verlet = p->nc_verlet > 0 ? p->nc_verlet : sys->nc;
  long len = (long) p->n * sys->s;
  sys->rk = (double *) calloc((size_t) len, sizeof(double));
  sys->af = (double *) calloc((size_t) p->n, sizeof(double));
  sys->card = (double *) calloc((size_t) p->n, sizeof(double));
  sys->caf = (double *) calloc((size_t) p->n, sizeof(double));
  sys->nat_freq = (double *) calloc((size_t) p->n, sizeof(double));
  sys->pll = (int *) calloc((size_t) p->n, sizeof(int));
  int maxc = sys->nc > sys->nc_verlet ? sys->nc : sys->nc_verlet;
  sys->cell_off = (int *) calloc((size_t) maxc * maxc + 1, sizeof(int));
  sys->cell_mem = (int *) calloc((size_t) p->n, sizeof(int));
  sys->verlet = (ilist *) calloc((size_t) p->n, sizeof(ilist));
  sys->should_update_lists = 1; /* ParticleSystemFirstOrder.cpp:63 */
  return sys;
}

void spo_destroy(spo_system *sys)
{
  if (!sys) return;
  free(sys->rk);
  free(sys->af);
  free(sys->card);
  free(sys->caf);
  free(sys->nat_freq);
  free(sys->pll);
  free(sys->cell_off);
  free(sys->cell_mem);
  for (int i = 0; i < sys->p.n; ++i) free(sys->verlet[i].data);
  free(sys->verlet);
  free(sys);
}

void spo_set_higher_order(spo_system *sys, int on)
{
  sys->higher_order = on;
}

void spo_set_natural_frequencies(spo_system *sys, const double *freqs)
{
  memcpy(sys->nat_freq, freqs, (size_t) sys->p.n * sizeof(double));
}

/* ------------------------------------------------------------ helpers */

/* rk_system_state = system_state + k_coef * dt * k_prev
 * (ParticleSystemFirstOrder.cpp:175-184; ParticleSystemSecondOrder.cpp:289-300). */
static void stage_state(spo_system *sys, const double *state, const double *k_prev, double k_coef, double dt)
{
  long len = (long) sys->p.n * sys->s;
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (long q = 0; q < len; ++q) sys->rk[q] = state[q] + k_coef * dt * k_prev[q];
}

/* Cell ids and the linked list (ParticleSystemFirstOrder.cpp:255-288,
 * ParticleSystemSecondOrder.cpp:303-339): a stable counting sort, so each
 * cell lists its particles in ascending index as the push_back loop does. */
static void build_cells(spo_system *sys, int nc)
{
  const int n = sys->p.n, s = sys->s;
  for (int i = 0; i < n; ++i)
  {
    double x = sys->rk[(long) s * i], y = sys->rk[(long) s * i + 1];
    if (sys->p.model == 1)
    {
      x = pbc_wrap(x);
      y = pbc_wrap(y);
    } else
    {
      wrap_if_outside(&x, &y);
    }
    sys->pll[i] = cell_coord(y, nc) * nc + cell_coord(x, nc);
  }
  int ncell = nc * nc;
  memset(sys->cell_off, 0, (size_t) (ncell + 1) * sizeof(int));
  for (int i = 0; i < n; ++i) sys->cell_off[sys->pll[i] + 1]++;
  for (int c = 0; c < ncell; ++c) sys->cell_off[c + 1] += sys->cell_off[c];
  int *fill = (int *) calloc((size_t) ncell, sizeof(int));
  for (int i = 0; i < n; ++i)
  {
    int c = sys->pll[i];
    sys->cell_mem[sys->cell_off[c] + fill[c]++] = i;
  }
  free(fill);
  sys->cells_built = ncell;
}

/* Position of particle i as the pair loops of each class see it. */
static inline void pos_i_for_cells(const spo_system *sys, int i, double *x, double *y)
{
  *x = sys->rk[(long) sys->s * i];
  *y = sys->rk[(long) sys->s * i + 1];
  if (sys->p.model == 1)
  {
    *x = pbc_wrap(*x);
    *y = pbc_wrap(*y);
  } else
  {
    wrap_if_outside(x, y);
  }
}

/* First-order pair term (ParticleSystemFirstOrderPtr.cpp:404-415). */
static inline void pair_first(const spo_system *sys, double phi_i, double omega_i, double phi_j, double omega_j,
                              double *af, double *card, double *caf)
{
  *af += sin(phi_j - phi_i) * sys->cos_alpha - cos(phi_j - phi_i) * sys->sin_alpha;
  *card += 1.0;
  if (sys->higher_order)
  {
    *caf += (omega_j - omega_i) * (cos(phi_j - phi_i) * sys->cos_alpha + sin(phi_j - phi_i) * sys->sin_alpha);
  }
}

/* Second-order pair term (ParticleSystemSecondOrder.cpp:160-161).  The
 * complementary force has no second-order reference code; it is the
 * first-order one (ParticleSystemFirstOrderPtr.cpp:409-414) with the
 * second-order sin(phi_j - phi_i - alpha) convention. */
static inline void pair_second(const spo_system *sys, double phi_i, double omega_i, double phi_j, double omega_j,
                               double *af, double *card, double *caf)
{
  *af += sin(phi_j - phi_i - sys->p.alpha);
  *card += 1.0;
  if (sys->higher_order) *caf += (omega_j - omega_i) * cos(phi_j - phi_i - sys->p.alpha);
}

/* Output of one particle (ParticleSystemFirstOrder.cpp:220-226,
 * ParticleSystemFirstOrderPtr.cpp:419-429, ParticleSystemSecondOrder.cpp:166-175).
 * k_next[ii+3] / [ii+5] is left untouched when particle i has no neighbour. */
static inline void write_k(const spo_system *sys, int i, const double *st, double af, double card, double caf,
                           double *k_next)
{
  long ii = (long) sys->s * i;
  const spo_params *p = &sys->p;
  if (p->model == 1)
  {
    double phi_i = st[2], omega_i = st[3];
    k_next[ii] = p->v0 * cos(phi_i);
    k_next[ii + 1] = p->v0 * sin(phi_i);
    k_next[ii + 2] = omega_i;
    if (card != 0.0)
    {
      k_next[ii + 3] = -p->xi * omega_i + p->sigma * af / card;
      if (sys->higher_order) caf *= p->sigma / card;
    }
  } else
  {
    double v_x_i = st[2], v_y_i = st[3], phi_i = st[4], omega_i = st[5];
    k_next[ii] = v_x_i;
    k_next[ii + 1] = v_y_i;
    k_next[ii + 2] = -p->xi_r * v_x_i + p->v0 * cos(phi_i);
    k_next[ii + 3] = -p->xi_r * v_y_i + p->v0 * sin(phi_i);
    k_next[ii + 4] = omega_i;
    if (card != 0.0)
    {
      k_next[ii + 5] = -p->xi_phi * omega_i + p->sigma * af / card;
      if (sys->higher_order) caf *= p->sigma / card;
    }
  }
  sys->af[i] = af;
  sys->card[i] = card;
  if (sys->higher_order) sys->caf[i] = caf;
}

static inline int phi_index(const spo_system *sys)
{
  return sys->p.model == 1 ? 2 : 4;
}

static void reset_sums(spo_system *sys)
{
  memset(sys->af, 0, (size_t) sys->p.n * sizeof(double));
  memset(sys->card, 0, (size_t) sys->p.n * sizeof(double));
  if (sys->higher_order) memset(sys->caf, 0, (size_t) sys->p.n * sizeof(double));
}

/* ---------------------------------------------------------- all pairs */

/* EvaluateInteractionsWithAllPairs: first order
 * (ParticleSystemFirstOrder.cpp:162-228; the MPI class additionally wraps x_i,
 * ParticleSystemFirstOrderPtr.cpp:263-266), second order
 * (ParticleSystemSecondOrder.cpp:116-177). */
static void rhs_all_pairs(spo_system *sys, double *k_next)
{
  const int n = sys->p.n, s = sys->s, ip = phi_index(sys);
  reset_sums(sys);
#pragma omp parallel for num_threads(g_threads) schedule(dynamic, 16)
  for (int i = 0; i < n; ++i)
  {
    const double *st = sys->rk + (long) s * i;
    double x_i = st[0], y_i = st[1], phi_i = st[ip], omega_i = st[ip + 1];
    if (sys->p.model == 1 && sys->p.flavor == 1)
    {
      x_i = pbc_wrap(x_i);
      y_i = pbc_wrap(y_i);
    }
    double af = 0.0, card = 0.0, caf = 0.0;
    for (int j = 0; j < n; ++j)
    {
      if (j == i) continue;
      const double *sj = sys->rk + (long) s * j;
      double dx, dy;
      if (sys->p.model == 1)
      {
        dx = pbc_class_c(sj[0] - x_i);
        dy = pbc_class_c(sj[1] - y_i);
      } else
      {
        dx = pbc_class_a(sj[0] - x_i);
        dy = pbc_class_a(sj[1] - y_i);
      }
      double dr2 = dx * dx + dy * dy;
      if (dr2 <= sys->rho_squared)
      {
        if (sys->p.model == 1) pair_first(sys, phi_i, omega_i, sj[ip], sj[ip + 1], &af, &card, &caf);
        else pair_second(sys, phi_i, omega_i, sj[ip], sj[ip + 1], &af, &card, &caf);
      }
    }
    write_k(sys, i, st, af, card, caf, k_next);
  }
}

/* --------------------------------------------------------- linked list */

/* EvaluateInteractionsWithLinkedList (ParticleSystemFirstOrder.cpp:231-353,
 * ParticleSystemFirstOrderPtr.cpp:318-468, ParticleSystemSecondOrder.cpp:276-409). */
static void rhs_linked_list(spo_system *sys, double *k_next)
{
  const int n = sys->p.n, s = sys->s, ip = phi_index(sys), nc = sys->nc;
  reset_sums(sys);
  build_cells(sys, nc);
#pragma omp parallel for num_threads(g_threads) schedule(dynamic, 64)
  for (int i = 0; i < n; ++i)
  {
    const double *st = sys->rk + (long) s * i;
    double x_i, y_i;
    pos_i_for_cells(sys, i, &x_i, &y_i);
    double phi_i = st[ip], omega_i = st[ip + 1];
    int cx = cell_coord(x_i, nc), cy = cell_coord(y_i, nc);
    double af = 0.0, card = 0.0, caf = 0.0;
    for (int c = 0; c < 9; ++c)
    {
      int jx = adjust_cell(cx + kStencil[c][0], nc), jy = adjust_cell(cy + kStencil[c][1], nc);
      int jc = jy * nc + jx;
      for (int m = sys->cell_off[jc]; m < sys->cell_off[jc + 1]; ++m)
      {
        int j = sys->cell_mem[m];
        if (j == i) continue;
        const double *sj = sys->rk + (long) s * j;
        double dx, dy;
        if (sys->p.model == 1)
        {
          dx = pbc_class_c(sj[0] - x_i);
          dy = pbc_class_c(sj[1] - y_i);
        } else
        {
          double x_j = sj[0], y_j = sj[1];
          wrap_if_outside(&x_j, &y_j);
          dx = pbc_class_a(x_j - x_i);
          dy = pbc_class_a(y_j - y_i);
        }
        double dr2 = dx * dx + dy * dy;
        if (dr2 <= sys->rho_squared)
        {
          if (sys->p.model == 1) pair_first(sys, phi_i, omega_i, sj[ip], sj[ip + 1], &af, &card, &caf);
          else pair_second(sys, phi_i, omega_i, sj[ip], sj[ip + 1], &af, &card, &caf);
        }
      }
    }
    write_k(sys, i, st, af, card, caf, k_next);
  }
}

/* ------------------------------------------------------------- Verlet */

static void clear_verlet(spo_system *sys)
{
  for (int i = 0; i < sys->p.n; ++i) sys->verlet[i].len = 0;
}

/* Verlet rebuild with an O(N^2) scan (ParticleSystemFirstOrder.cpp:376-422):
 * unwrapped stage positions, ClassC distance, r <= r_max.  For the
 * second-order model (no reference code) the positions are wrapped if they
 * left the box and the ClassA distance is used, as in its other routines. */
static void build_verlet_all_pairs(spo_system *sys)
{
  const int n = sys->p.n, s = sys->s;
  const double rmax2 = sys->p.r_max * sys->p.r_max;
  clear_verlet(sys);
#pragma omp parallel for num_threads(g_threads) schedule(dynamic, 16)
  for (int i = 0; i < n; ++i)
  {
    double x_i = sys->rk[(long) s * i], y_i = sys->rk[(long) s * i + 1];
    if (sys->p.model == 2) wrap_if_outside(&x_i, &y_i);
    for (int j = 0; j < n; ++j)
    {
      if (j == i) continue;
      double x_j = sys->rk[(long) s * j], y_j = sys->rk[(long) s * j + 1], dx, dy;
      if (sys->p.model == 1)
      {
        dx = pbc_class_c(x_j - x_i);
        dy = pbc_class_c(y_j - y_i);
      } else
      {
        wrap_if_outside(&x_j, &y_j);
        dx = pbc_class_a(x_j - x_i);
        dy = pbc_class_a(y_j - y_i);
      }
      if (dx * dx + dy * dy <= rmax2) ilist_push(&sys->verlet[i], j);
    }
  }
}

/* Verlet rebuild from the cell list (ParticleSystemFirstOrder.cpp:501-592,
 * ParticleSystemFirstOrderPtr.cpp:759-859): cells of the Verlet grid, wrapped
 * x_i against unwrapped x_j (ClassC) for the first-order model.  The
 * second-order restatement wraps both if they left the box (ClassA). */
static void build_verlet_cells(spo_system *sys)
{
  const int n = sys->p.n, s = sys->s, nc = sys->nc_verlet;
  const double rmax2 = sys->p.r_max * sys->p.r_max;
  build_cells(sys, nc);
  clear_verlet(sys);
#pragma omp parallel for num_threads(g_threads) schedule(dynamic, 64)
  for (int i = 0; i < n; ++i)
  {
    double x_i, y_i;
    pos_i_for_cells(sys, i, &x_i, &y_i);
    int cx = cell_coord(x_i, nc), cy = cell_coord(y_i, nc);
    for (int c = 0; c < 9; ++c)
    {
      int jx = adjust_cell(cx + kStencil[c][0], nc), jy = adjust_cell(cy + kStencil[c][1], nc);
      int jc = jy * nc + jx;
      for (int m = sys->cell_off[jc]; m < sys->cell_off[jc + 1]; ++m)
      {
        int j = sys->cell_mem[m];
        if (j == i) continue;
        double x_j = sys->rk[(long) s * j], y_j = sys->rk[(long) s * j + 1], dx, dy;
        if (sys->p.model == 1)
        {
          dx = pbc_class_c(x_j - x_i);
          dy = pbc_class_c(y_j - y_i);
        } else
        {
          wrap_if_outside(&x_j, &y_j);
          dx = pbc_class_a(x_j - x_i);
          dy = pbc_class_a(y_j - y_i);
        }
        if (dx * dx + dy * dy <= rmax2) ilist_push(&sys->verlet[i], j);
      }
    }
  }
}

/* Pair loop over the Verlet list (ParticleSystemFirstOrder.cpp:594-648,
 * ParticleSystemFirstOrderPtr.cpp:861-930): unwrapped positions for the first
 * order; the second-order restatement wraps positions that left the box. */
static void rhs_verlet_pairs(spo_system *sys, double *k_next)
{
  const int n = sys->p.n, s = sys->s, ip = phi_index(sys);
  reset_sums(sys);
#pragma omp parallel for num_threads(g_threads) schedule(dynamic, 64)
  for (int i = 0; i < n; ++i)
  {
    const double *st = sys->rk + (long) s * i;
    double x_i = st[0], y_i = st[1], phi_i = st[ip], omega_i = st[ip + 1];
    if (sys->p.model == 2) wrap_if_outside(&x_i, &y_i);
    double af = 0.0, card = 0.0, caf = 0.0;
    const ilist *l = &sys->verlet[i];
    for (int m = 0; m < l->len; ++m)
    {
      int j = l->data[m];
      if (j == i) continue;
      const double *sj = sys->rk + (long) s * j;
      double dx, dy;
      if (sys->p.model == 1)
      {
        dx = pbc_class_c(sj[0] - x_i);
        dy = pbc_class_c(sj[1] - y_i);
      } else
      {
        double x_j = sj[0], y_j = sj[1];
        wrap_if_outside(&x_j, &y_j);
        dx = pbc_class_a(x_j - x_i);
        dy = pbc_class_a(y_j - y_i);
      }
      double dr2 = dx * dx + dy * dy;
      if (dr2 <= sys->rho_squared)
      {
        if (sys->p.model == 1) pair_first(sys, phi_i, omega_i, sj[ip], sj[ip + 1], &af, &card, &caf);
        else pair_second(sys, phi_i, omega_i, sj[ip], sj[ip + 1], &af, &card, &caf);
      }
    }
    write_k(sys, i, st, af, card, caf, k_next);
  }
}

/* --------------------------------------------------------- global field */

/* EvaluateInteractionsWithGlobalPolarOrderField, first order only:
 * ParticleSystemFirstOrder.cpp:122-159 (serial class) and
 * ParticleSystemFirstOrderPtr.cpp:155-223 (MPI class, with the weighted field
 * and the complementary force, including its use of arg(weighted field) in
 * the last sine at :219, reproduced as written). */
static void rhs_global_field(spo_system *sys, double *k_next)
{
  const int n = sys->p.n, s = sys->s;
  const spo_params *p = &sys->p;
  double pre = 0.0, pim = 0.0, wre = 0.0, wim = 0.0;
  for (int i = 0; i < n; ++i)
  {
    double phi_i = sys->rk[(long) s * i + 2], omega_i = sys->rk[(long) s * i + 3];
    double c = cos(phi_i), sn = sin(phi_i);
    pre += c;
    pim += sn;
    wre += omega_i * c;
    wim += omega_i * sn;
  }
  pre /= n;
  pim /= n;
  wre /= n;
  wim /= n;
  const double pabs = hypot(pre, pim), parg = atan2(pim, pre);
  const double wabs = hypot(wre, wim), warg = atan2(wim, wre);
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int i = 0; i < n; ++i)
  {
    long ii = (long) s * i;
    double phi_i = sys->rk[ii + 2], omega_i = sys->rk[ii + 3];
    k_next[ii] = p->v0 * cos(phi_i);
    k_next[ii + 1] = p->v0 * sin(phi_i);
    k_next[ii + 2] = omega_i;
    k_next[ii + 3] = -p->xi * omega_i + sys->nat_freq[i]
        + p->sigma * pabs * (sin(parg - phi_i) * sys->cos_alpha - cos(parg - phi_i) * sys->sin_alpha);
    if (p->flavor == 1 && sys->higher_order)
    {
      sys->caf[i] = p->sigma * (wabs * (cos(warg - phi_i) * sys->cos_alpha + sin(warg - phi_i) * sys->sin_alpha)
          - omega_i * pabs * (cos(parg - phi_i) * sys->cos_alpha + sin(warg - phi_i) * sys->sin_alpha));
    }
  }
}

/* ------------------------------------------------------------ dispatch */

int spo_evaluate(spo_system *sys, int variant, const double *state, const double *k_prev, double *k_next,
                 double k_coef, double dt)
{
  const spo_params *p = &sys->p;
  if (variant == SPO_DISPATCH)
  {
    if (p->model == 1)
    {
      /* ParticleSystemFirstOrder.cpp:96-111 */
      if (p->rho >= M_SQRT1_2) variant = SPO_GLOBAL_FIELD;
      else if (p->rho <= 0.25) variant = SPO_LINKED_LIST_VERLET;
      else if (p->rho <= 0.5) variant = SPO_VERLET;
      else variant = SPO_ALL_PAIRS;
    } else
    {
      /* ParticleSystemSecondOrder.cpp:91-98 */
      variant = (p->rho <= 0.25) ? SPO_LINKED_LIST : SPO_ALL_PAIRS;
    }
  }
  if (variant == SPO_GLOBAL_FIELD && p->model != 1) return -1;
  if (variant < SPO_ALL_PAIRS || variant > SPO_GLOBAL_FIELD) return -1;
  stage_state(sys, state, k_prev, k_coef, dt);
  switch (variant)
  {
    case SPO_ALL_PAIRS:
      rhs_all_pairs(sys, k_next);
      break;
    case SPO_LINKED_LIST:
      rhs_linked_list(sys, k_next);
      break;
    case SPO_VERLET:
      if (sys->should_update_lists)
      {
        build_verlet_all_pairs(sys);
        sys->should_update_lists = 0;
      }
      rhs_verlet_pairs(sys, k_next);
      sys->uses_verlet_list = 1;
      break;
    case SPO_LINKED_LIST_VERLET:
      if (sys->should_update_lists)
      {
        build_verlet_cells(sys);
        sys->should_update_lists = 0;
      }
      rhs_verlet_pairs(sys, k_next);
      sys->uses_verlet_list = 1;
      break;
    case SPO_GLOBAL_FIELD:
      rhs_global_field(sys, k_next);
      break;
  }
  return 0;
}

void spo_get_complementary_force(const spo_system *sys, double *out)
{
  memcpy(out, sys->caf, (size_t) sys->p.n * sizeof(double));
}

/* CalculateMaxDisplacement (ParticleSystemFirstOrder.cpp:670-696). */
void spo_calculate_max_displacement(spo_system *sys, const double *td)
{
  double max2 = 0.0;
  for (int i = 0; i < sys->p.n; ++i)
  {
    double dx = td[(long) sys->s * i], dy = td[(long) sys->s * i + 1];
    double d2 = dx * dx + dy * dy;
    if (max2 < d2) max2 = d2;
  }
  sys->accumulated_displacement += sqrt(max2);
  int flag = 0;
  if (sys->accumulated_displacement > 0.5 * (sys->p.r_max - sys->r_min))
  {
    sys->accumulated_displacement = 0.0;
    flag = 1;
  }
  sys->should_update_lists = flag;
}

double spo_accumulated_displacement(const spo_system *sys)
{
  return sys->accumulated_displacement;
}

int spo_should_update_lists(const spo_system *sys)
{
  return sys->should_update_lists;
}

void spo_set_should_update_lists(spo_system *sys, int flag)
{
  sys->should_update_lists = flag;
}

int spo_uses_verlet_list(const spo_system *sys)
{
  return sys->uses_verlet_list;
}

int spo_num_cells_per_side(const spo_system *sys, int verlet_grid)
{
  return verlet_grid ? sys->nc_verlet : sys->nc;
}

void spo_get_pre_linked_list(const spo_system *sys, int *out)
{
  memcpy(out, sys->pll, (size_t) sys->p.n * sizeof(int));
}

long spo_get_cells(const spo_system *sys, int *offsets, int *members)
{
  if (offsets) memcpy(offsets, sys->cell_off, (size_t) (sys->cells_built + 1) * sizeof(int));
  if (members) memcpy(members, sys->cell_mem, (size_t) sys->p.n * sizeof(int));
  return sys->cells_built;
}

long spo_get_verlet(const spo_system *sys, int *offsets, int *entries)
{
  long total = 0;
  for (int i = 0; i < sys->p.n; ++i)
  {
    if (offsets) offsets[i] = (int) total;
    if (entries) memcpy(entries + total, sys->verlet[i].data, (size_t) sys->verlet[i].len * sizeof(int));
    total += sys->verlet[i].len;
  }
  if (offsets) offsets[sys->p.n] = (int) total;
  return total;
}

/* ------------------------------------------------------------ steppers */

spo_stepper *spo_stepper_create(int n, int s)
{
  spo_stepper *st = (spo_stepper *) calloc(1, sizeof(spo_stepper));
  size_t len = (size_t) n * s;
  st->n = n;
  st->s = s;
  st->k1 = (double *) calloc(len, sizeof(double));
  st->k2 = (double *) calloc(len, sizeof(double));
  st->k3 = (double *) calloc(len, sizeof(double));
  st->k4 = (double *) calloc(len, sizeof(double));
  st->td = (double *) calloc(len, sizeof(double));
  st->det = (double *) calloc(len, sizeof(double));
  st->stoch = (double *) calloc(len, sizeof(double));
  return st;
}

void spo_stepper_destroy(spo_stepper *st)
{
  if (!st) return;
  free(st->k1);
  free(st->k2);
  free(st->k3);
  free(st->k4);
  free(st->td);
  free(st->det);
  free(st->stoch);
  free(st);
}

int spo_normals_per_particle(int model, int stepper)
{
  /* stepper: 0 RK4, 1 stochastic Euler, 2 stochastic Runge-Kutta */
  if (stepper == 0) return 0;
  if (stepper == 1) return model == 1 ? 1 : 3;
  return model == 1 ? 2 : 6;
}

/* RungeKutta4Stepper::DoStep (Steppers/RungeKutta4Stepper.cpp:29-64, :66-101;
 * RungeKutta4StepperPtr.cpp:31-78).  k buffers persist across steps, so a
 * component the RHS leaves unwritten keeps its previous-step value. */
int spo_rk4_step(spo_system *sys, spo_stepper *st, int variant, double *state, double t, double dt)
{
  (void) t;
  if (spo_evaluate(sys, variant, state, st->k1, st->k1, 0.0, dt)) return -1;
  spo_evaluate(sys, variant, state, st->k1, st->k2, 0.5, dt);
  spo_evaluate(sys, variant, state, st->k2, st->k3, 0.5, dt);
  spo_evaluate(sys, variant, state, st->k3, st->k4, 1.0, dt);
  long len = (long) st->n * st->s;
  for (long q = 0; q < len; ++q)
  {
    st->td[q] = (st->k1[q] + 2.0 * st->k2[q] + 2.0 * st->k3[q] + st->k4[q]) * dt / 6.0;
    state[q] += st->td[q];
  }
  if (sys->uses_verlet_list) spo_calculate_max_displacement(sys, st->td);
  return 0;
}

/* Stochastic Euler.
 * Second order: StochasticEulerStepper::DoStep (Steppers/StochasticEulerStepper.hpp:33-51)
 *   with ParticleSystemSecondOrder::AddNoise (ParticleSystemSecondOrder.cpp:439-451):
 *   normals per particle in the order (r_x, r_y, phi) -> components 2, 3, 5.
 * First order: StochasticEulerStepperPtr::DoStep (StochasticEulerStepperPtr.hpp:40-73):
 *   one normal per particle -> omega.
 * The reference's second-order stepper has no Verlet trigger (the model has no
 * Verlet routine); the restated second-order Verlet calls it with the step's
 * increment, as the first-order steppers do. */
int spo_se_step(spo_system *sys, spo_stepper *st, int variant, double *state, double t, double dt,
                const double *normals)
{
  (void) t;
  const int n = st->n, s = st->s;
  long len = (long) n * s;
  memset(st->det, 0, (size_t) len * sizeof(double));
  if (spo_evaluate(sys, variant, state, st->det, st->det, 0.0, dt)) return -1;
  if (sys->p.model == 2)
  {
    memset(st->stoch, 0, (size_t) len * sizeof(double));
    const double intensity_r = sqrt(2.0 * sys->p.D_r), intensity_phi = sqrt(2.0 * sys->p.D_phi);
    for (int i = 0; i < n; ++i)
    {
      st->stoch[(long) s * i + 2] = intensity_r * normals[3L * i];
      st->stoch[(long) s * i + 3] = intensity_r * normals[3L * i + 1];
      st->stoch[(long) s * i + 5] = intensity_phi * normals[3L * i + 2];
    }
    for (long q = 0; q < len; ++q)
    {
      st->td[q] = dt * st->det[q] + sqrt(dt) * st->stoch[q];
      state[q] += dt * st->det[q] + sqrt(dt) * st->stoch[q];
    }
  } else
  {
    const double intensity_phi = sqrt(2.0 * sys->p.D_phi);
    for (int i = 0; i < n; ++i)
    {
      double delta_W_phi = sqrt(dt) * normals[i];
      long ii = (long) s * i;
      st->td[ii] = st->det[ii] * dt;
      st->td[ii + 1] = st->det[ii + 1] * dt;
      st->td[ii + 2] = st->det[ii + 2] * dt;
      st->td[ii + 3] = st->det[ii + 3] * dt + intensity_phi * delta_W_phi;
      state[ii] += st->td[ii];
      state[ii + 1] += st->td[ii + 1];
      state[ii + 2] += st->td[ii + 2];
      state[ii + 3] += st->td[ii + 3];
    }
  }
  if (sys->uses_verlet_list) spo_calculate_max_displacement(sys, st->td);
  return 0;
}

/* Strong order 1.5 stochastic Taylor scheme.
 * First order: StochasticRungeKuttaStepperPtr::DoStep
 *   (Steppers/StochasticRungeKuttaStepperPtr.hpp:40-76); normals (U1, U2) per particle.
 * Second order (no reference code; derived with the same scheme for additive
 * noise, Kloeden & Platen sec. 10.4, which the reference cites at :17-20):
 *   drift a = (v_x, v_y, -xi_r v_x + v0 cos phi, -xi_r v_y + v0 sin phi, omega, -xi_phi omega + sigma F),
 *   noise b_r = sqrt(2 D_r) on v_x, v_y and b_phi = sqrt(2 D_phi) on omega,
 *   three Wiener processes with normals (U1, U2) each, per particle in the
 *   order (v_x, v_y, omega).  With dW = U1 sqrt(dt), dZ = dt^1.5 (U1 + U2/sqrt3)/2:
 *     x   += a_x dt + a_vx dt^2/2 + b_r dZ_x
 *     y   += a_y dt + a_vy dt^2/2 + b_r dZ_y
 *     v_x += a_vx dt + (-xi_r a_vx - v0 sin(phi) a_phi) dt^2/2 + b_r (dW_x - xi_r dZ_x)
 *     v_y += a_vy dt + (-xi_r a_vy + v0 cos(phi) a_phi) dt^2/2 + b_r (dW_y - xi_r dZ_y)
 *     phi += a_phi dt + a_omega dt^2/2 + b_phi dZ_w
 *     om  += a_omega dt + (C - xi_phi a_omega) dt^2/2 + b_phi (dW_w - xi_phi dZ_w)
 *   with C the complementary alignment force sigma/N_i sum_j (om_j - om_i) cos(phi_j - phi_i - alpha),
 *   the second-order analogue of the first-order term at :66-67. */
int spo_srk_step(spo_system *sys, spo_stepper *st, int variant, double *state, double t, double dt,
                 const double *normals)
{
  (void) t;
  const int n = st->n, s = st->s;
  long len = (long) n * s;
  double *d = st->det, *td = st->td;
  memset(d, 0, (size_t) len * sizeof(double));
  sys->higher_order = 1;
  if (spo_evaluate(sys, variant, state, d, d, 0.0, dt)) return -1;
  const double *caf = sys->caf;
  const spo_params *p = &sys->p;
  if (p->model == 1)
  {
    double noise = p->D_phi, friction = p->xi;
    for (int i = 0; i < n; ++i)
    {
      double U_1 = normals[2L * i], U_2 = normals[2L * i + 1];
      double delta_W_i = U_1 * sqrt(dt);
      double delta_Z_i = 0.5 * pow(dt, 1.5) * (U_1 + 1.0 / sqrt(3.0) * U_2);
      long ii = (long) s * i;
      td[ii] = d[ii] * dt - 0.5 * d[ii + 2] * d[ii + 1] * dt * dt;
      td[ii + 1] = d[ii + 1] * dt + 0.5 * d[ii + 2] * d[ii] * dt * dt;
      td[ii + 2] = d[ii + 2] * dt + 0.5 * d[ii + 3] * dt * dt + sqrt(2.0 * noise) * delta_Z_i;
      td[ii + 3] = d[ii + 3] * dt + 0.5 * (caf[i] - friction * d[ii + 3]) * dt * dt
          + sqrt(2.0 * noise) * (delta_W_i - friction * delta_Z_i);
      state[ii] += td[ii];
      state[ii + 1] += td[ii + 1];
      state[ii + 2] += td[ii + 2];
      state[ii + 3] += td[ii + 3];
    }
  } else
  {
    const double b_r = sqrt(2.0 * p->D_r), b_phi = sqrt(2.0 * p->D_phi);
    const double sqdt = sqrt(dt), dt15 = pow(dt, 1.5), inv_sqrt3 = 1.0 / sqrt(3.0);
    for (int i = 0; i < n; ++i)
    {
      const double *u = normals + 6L * i;
      double dWx = u[0] * sqdt, dZx = 0.5 * dt15 * (u[0] + inv_sqrt3 * u[1]);
      double dWy = u[2] * sqdt, dZy = 0.5 * dt15 * (u[2] + inv_sqrt3 * u[3]);
      double dWw = u[4] * sqdt, dZw = 0.5 * dt15 * (u[4] + inv_sqrt3 * u[5]);
      long ii = (long) s * i;
      double phi = state[ii + 4];
      double cphi = cos(phi), sphi = sin(phi);
      td[ii] = d[ii] * dt + 0.5 * d[ii + 2] * dt * dt + b_r * dZx;
      td[ii + 1] = d[ii + 1] * dt + 0.5 * d[ii + 3] * dt * dt + b_r * dZy;
      td[ii + 2] = d[ii + 2] * dt + 0.5 * (-p->xi_r * d[ii + 2] - p->v0 * sphi * d[ii + 4]) * dt * dt
          + b_r * (dWx - p->xi_r * dZx);
      td[ii + 3] = d[ii + 3] * dt + 0.5 * (-p->xi_r * d[ii + 3] + p->v0 * cphi * d[ii + 4]) * dt * dt
          + b_r * (dWy - p->xi_r * dZy);
      td[ii + 4] = d[ii + 4] * dt + 0.5 * d[ii + 5] * dt * dt + b_phi * dZw;
      td[ii + 5] = d[ii + 5] * dt + 0.5 * (caf[i] - p->xi_phi * d[ii + 5]) * dt * dt
          + b_phi * (dWw - p->xi_phi * dZw);
      for (int q = 0; q < 6; ++q) state[ii + q] += td[ii + q];
    }
  }
  if (sys->uses_verlet_list) spo_calculate_max_displacement(sys, td);
  return 0;
}

/* ------------------------------------------------------- observers */

/* BinaryObserver*::SaveSummaryStatistics (BinaryObserverFirstOrder.cpp:125-142,
 * BinaryObserverSecondOrder.cpp:121-138) accumulate in complex<float>; this
 * restatement accumulates in FP64.  The velocity polar order parameter of the
 * second-order model has no reference code. */
void spo_order_parameters(int model, int n, const double *state, double *out)
{
  const int s = model == 1 ? 4 : 6, ip = model == 1 ? 2 : 4;
  double re = 0.0, im = 0.0, vre = 0.0, vim = 0.0;
  for (int i = 0; i < n; ++i)
  {
    double phi = state[(long) s * i + ip];
    re += cos(phi);
    im += sin(phi);
    if (model == 2)
    {
      double vx = state[(long) s * i + 2], vy = state[(long) s * i + 3];
      double v = sqrt(vx * vx + vy * vy);
      if (v > 0.0)
      {
        vre += vx / v;
        vim += vy / v;
      }
    }
  }
  re /= n;
  im /= n;
  out[0] = sqrt(re * re + im * im);
  out[1] = atan2(im, re);
  if (model == 2)
  {
    vre /= n;
    vim /= n;
    out[2] = sqrt(vre * vre + vim * vim);
    out[3] = atan2(vim, vre);
  } else
  {
    out[2] = out[0];
    out[3] = out[1];
  }
}

/* ---------------------------------------------------------------- Philox */

/* Philox4x32-10 (Salmon, Moraes, Dror & Shaw, SC'11) and a Box-Muller
 * transform; used only by the CPU-baseline leg to draw its own noise. */
static void philox4x32_10(uint32_t ctr[4], const uint32_t key_in[2])
{
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; ++r)
  {
    uint64_t p0 = (uint64_t) 0xD2511F53u * ctr[0];
    uint64_t p1 = (uint64_t) 0xCD9E8D57u * ctr[2];
    uint32_t hi0 = (uint32_t) (p0 >> 32), lo0 = (uint32_t) p0;
    uint32_t hi1 = (uint32_t) (p1 >> 32), lo1 = (uint32_t) p1;
    uint32_t n0 = hi1 ^ ctr[1] ^ k0, n2 = hi0 ^ ctr[3] ^ k1;
    ctr[0] = n0;
    ctr[1] = lo1;
    ctr[2] = n2;
    ctr[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

void spo_philox_normals(unsigned long long seed, unsigned long long step, int stream, long count, double *out)
{
  const uint32_t key[2] = {(uint32_t) seed, (uint32_t) (seed >> 32)};
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (long b = 0; b < (count + 3) / 4; ++b)
  {
    uint32_t ctr[4] = {(uint32_t) b, (uint32_t) step, (uint32_t) (step >> 32), (uint32_t) stream};
    philox4x32_10(ctr, key);
    for (int h = 0; h < 2; ++h)
    {
      double u1 = ((double) ctr[2 * h] + 0.5) * (1.0 / 4294967296.0);
      double u2 = ((double) ctr[2 * h + 1] + 0.5) * (1.0 / 4294967296.0);
      double r = sqrt(-2.0 * log(u1));
      double a = 6.283185307179586 * u2;
      long q = 4 * b + 2 * h;
      if (q < count) out[q] = r * cos(a);
      if (q + 1 < count) out[q + 1] = r * sin(a);
    }
  }
}
