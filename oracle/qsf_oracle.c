/*
 * qsf_oracle.c -- CPU restatement of QSF's split-operator time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: tests/, the smoke check in
 * __graft_entry__.py and the cpu_baseline / reference legs of bench.py are the only
 * code that may load it.  The product path (qsf_gb300/, libqsfgpu.so) never links,
 * loads or falls back to it.
 *
 * Every function restates one piece of the reference (QSF-physics/QSF, header-only
 * C++), citing the file:line it follows.  Arithmetic is FP64 / complex128 throughout,
 * summations run in the reference's flat C order so that values agree with the
 * reference to the last few ulps.
 *
 * The DFT is FFTW's job in the reference (un-vendored, version unpinned).  Here it is
 * a mixed-radix Stockham FFT (radices 4, 2, 3, 5 and a direct DFT for other primes)
 * written from the textbook definition  X_k = sum_j x_j exp(sign * 2 pi i j k / n),
 * unnormalised, sign = -1 forward (FFTW_FORWARD) and +1 backward (FFTW_BACKWARD).
 * Twiddles come from long-double sin/cos so that they are correctly rounded doubles.
 */
#define _USE_MATH_DEFINES
#include <math.h>
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#include <stdlib.h>
#include <string.h>
#include <stdint.h>

typedef struct { double re, im; } orc_cx;

/* ------------------------------------------------------------------ FFT */

typedef struct {
  long n;
  int nstage;
  int radix[64];
  orc_cx* w; /* w[j] = exp(-2 pi i j / n), j < n */
} orc_fft_plan;

static orc_fft_plan* g_plans[64];
static int g_nplans = 0;

static orc_fft_plan* plan_get(long n) {
  for (int i = 0; i < g_nplans; ++i)
    if (g_plans[i]->n == n) return g_plans[i];
  orc_fft_plan* p = (orc_fft_plan*)calloc(1, sizeof(orc_fft_plan));
  p->n = n;
  long r = n;
  /* radix order: 4s first, then 2, 3, 5, then remaining primes */
  while (r % 4 == 0) { p->radix[p->nstage++] = 4; r /= 4; }
  while (r % 2 == 0) { p->radix[p->nstage++] = 2; r /= 2; }
  while (r % 3 == 0) { p->radix[p->nstage++] = 3; r /= 3; }
  while (r % 5 == 0) { p->radix[p->nstage++] = 5; r /= 5; }
  for (long f = 7; r > 1; f += 2)
    while (r % f == 0) { p->radix[p->nstage++] = (int)f; r /= f; }
  p->w = (orc_cx*)malloc(sizeof(orc_cx) * (size_t)n);
  const long double twopi = 6.283185307179586476925286766559005768L;
  for (long j = 0; j < n; ++j) {
    long double a = twopi * (long double)j / (long double)n;
    p->w[j].re = (double)cosl(a);
    p->w[j].im = -(double)sinl(a);
  }
  if (g_nplans < 64) g_plans[g_nplans++] = p;
  return p;
}

static inline orc_cx cmul(orc_cx a, orc_cx b) {
  orc_cx r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
  return r;
}

/* twiddle exp(sign*2 pi i t / n) from the table */
static inline orc_cx tw(const orc_fft_plan* p, long t, int sign) {
  orc_cx w = p->w[t % p->n];
  if (sign > 0) w.im = -w.im;
  return w;
}

/* One 1-D transform of x[0..n) (contiguous) using scratch y.  Stockham autosort:
 * pass with radix r and current sub-length ns reads x[j + q n/r], twiddles by
 * exp(sign 2 pi i (j mod ns) q / (ns r)), does an r-point DFT and writes
 * y[(j/ns) ns r + (j mod ns) + q ns]. */
static void fft_line(orc_cx* x, orc_cx* y, long n, int sign) {
  if (n <= 1) return;
  orc_fft_plan* p = plan_get(n);
  orc_cx* in = x;
  orc_cx* out = y;
  long ns = 1;
  /* butterfly buffers: on the stack for radices up to 64, else on the heap (a prime
   * length is one radix-n pass, a direct DFT, as FFTW plans any n) */
  int maxr = 0;
  for (int s = 0; s < p->nstage; ++s) maxr = p->radix[s] > maxr ? p->radix[s] : maxr;
  orc_cx vs[64], us[64];
  orc_cx* v = maxr <= 64 ? vs : (orc_cx*)malloc(sizeof(orc_cx) * (size_t)maxr);
  orc_cx* u = maxr <= 64 ? us : (orc_cx*)malloc(sizeof(orc_cx) * (size_t)maxr);
  for (int s = 0; s < p->nstage; ++s) {
    int r = p->radix[s];
    long nr = n / r;
    for (long j = 0; j < nr; ++j) {
      long jm = j % ns;
      for (int q = 0; q < r; ++q) {
        v[q] = in[j + q * nr];
        if (q && jm) v[q] = cmul(v[q], tw(p, jm * q * (n / (ns * r)), sign));
      }
      if (r == 2) {
        u[0].re = v[0].re + v[1].re; u[0].im = v[0].im + v[1].im;
        u[1].re = v[0].re - v[1].re; u[1].im = v[0].im - v[1].im;
      } else if (r == 4) {
        orc_cx a0 = {v[0].re + v[2].re, v[0].im + v[2].im};
        orc_cx a1 = {v[0].re - v[2].re, v[0].im - v[2].im};
        orc_cx a2 = {v[1].re + v[3].re, v[1].im + v[3].im};
        orc_cx a3 = {v[1].re - v[3].re, v[1].im - v[3].im};
        /* multiply a3 by sign*i */
        orc_cx b3 = sign < 0 ? (orc_cx){a3.im, -a3.re} : (orc_cx){-a3.im, a3.re};
        u[0].re = a0.re + a2.re; u[0].im = a0.im + a2.im;
        u[2].re = a0.re - a2.re; u[2].im = a0.im - a2.im;
        u[1].re = a1.re + b3.re; u[1].im = a1.im + b3.im;
        u[3].re = a1.re - b3.re; u[3].im = a1.im - b3.im;
      } else {
        /* direct r-point DFT */
        for (int k = 0; k < r; ++k) {
          orc_cx acc = v[0];
          for (int q = 1; q < r; ++q) {
            orc_cx t = cmul(v[q], tw(p, (long)((q * k) % r) * (n / r), sign));
            acc.re += t.re; acc.im += t.im;
          }
          u[k] = acc;
        }
      }
      long base = (j / ns) * ns * r + jm;
      for (int q = 0; q < r; ++q) out[base + q * ns] = u[q];
    }
    ns *= r;
    orc_cx* t = in; in = out; out = t;
  }
  if (in != x) memcpy(x, in, sizeof(orc_cx) * (size_t)n);
  if (v != vs) free(v);
  if (u != us) free(u);
}

/* In-place transform along the axes d with use[d] != 0 (all axes: use == NULL) of a
 * C-ordered array (last axis contiguous), last axis first. */
void orc_fft_axes(double* data, int dim, const long* n, const int* use, int sign) {
  orc_cx* a = (orc_cx*)data;
  long m = 1;
  for (int d = 0; d < dim; ++d) m *= n[d];
  long nmax = 1;
  for (int d = 0; d < dim; ++d) if (n[d] > nmax) nmax = n[d];
  orc_cx* line = (orc_cx*)malloc(sizeof(orc_cx) * (size_t)nmax);
  orc_cx* scr = (orc_cx*)malloc(sizeof(orc_cx) * (size_t)nmax);
  long stride = 1;
  for (int d = dim - 1; d >= 0; --d) {
    long nd = n[d];
    long outer = m / (nd * stride);
    if (use && !use[d]) {
      stride *= nd;
      continue;
    }
    for (long o = 0; o < outer; ++o)
      for (long in = 0; in < stride; ++in) {
        orc_cx* base = a + o * nd * stride + in;
        if (stride == 1) {
          fft_line(base, scr, nd, sign);
        } else {
          for (long k = 0; k < nd; ++k) line[k] = base[k * stride];
          fft_line(line, scr, nd, sign);
          for (long k = 0; k < nd; ++k) base[k * stride] = line[k];
        }
      }
    stride *= nd;
  }
  free(line);
  free(scr);
}

/* In-place N-D transform over all axes of a C-ordered array (last axis contiguous). */
void orc_fft_nd(double* data, int dim, const long* n, int sign) { orc_fft_axes(data, dim, n, NULL, sign); }

/* ------------------------------------------------------------------ grid */

enum { ORC_POT_EBERLY = 0, ORC_POT_ECKHARDT_SACHA = 1, ORC_POT_COULOMB = 2, ORC_POT_NONE = 3 };
enum { ORC_GAUGE_VELOCITY = 0, ORC_GAUGE_LENGTH = 1 };
enum { ORC_MODE_IM = 1, ORC_MODE_RE = 2 };
enum { ORC_REP_X = 1, ORC_REP_P = 2 };
enum { ORC_OP_IDENTITY = 0, ORC_OP_POTENTIAL = 1, ORC_OP_KINETIC = 2 };

typedef struct {
  int dim;
  long n[3];
  double dx[3];
  long m, n2[3], stride[3];
  double xmin[3], dp[3], inv_2dx[3], dV, dVm, inv_m;
  long nCAP; /* <= 0: no absorber */
  double eta;
  int pot;
  double NEcharge, EEcharge, Nsoft, Esoft;
  int gauge;
  int n_fields; /* coupling has this many fields; 0 -> coupling term is exactly 0 */
  int p_swap;   /* emulate the transposed P layout (coupling of axes 0 and 1 swapped) */
  int free_mask; /* region of a multi-region grid: axes kept in P space (bit d = axis d) */
  int multi;     /* multi-region grid: partial potentials, no absorber in evolve */
  int abs_kind;    /* 0 quartic CAP (absorbers.h), 1 cos^(1/8) mask (orc_grid_set_absorber) */
  double abs_rate; /* cos^(1/8) mask: applications per unit time (1 / mask_dt) */
} orc_grid;

/* coords.h:55-93 (CartesianGrid_::init), absorbers.h:27-33 (eta), potential.h:122-124 */
void orc_grid_init(orc_grid* g, int dim, const long* n, const double* dx, long nCAP, int pot,
                   double Ncharge, double Echarge, double Nsoft, double Esoft, int gauge,
                   int n_fields) {
  memset(g, 0, sizeof(*g));
  g->dim = dim;
  g->m = 1;
  for (int d = 0; d < dim; ++d) {
    g->n[d] = n[d];
    g->dx[d] = dx[d];
    g->n2[d] = n[d] / 2;
    g->m *= n[d];
  }
  g->inv_m = 1.0 / (double)g->m;
  g->dV = 1.0;
  for (int d = 0; d < dim; ++d) {
    g->dV *= dx[d];
    double L = dx[d] * (double)(n[d] - 1);
    g->xmin[d] = -0.5 * L;
    double inv_dx = 1.0 / dx[d];
    g->inv_2dx[d] = inv_dx / 2.0;
    g->dp[d] = 2.0 * M_PI / (double)n[d] / dx[d];
  }
  g->dVm = g->dV * g->inv_m;
  long s = 1;
  for (int d = dim - 1; d >= 0; --d) { g->stride[d] = s; s *= n[d]; }
  g->nCAP = nCAP;
  if (nCAP > 0) {
    double t = 3.0 / (double)nCAP;
    g->eta = t * (t * (t * t)); /* Power(3.0/nCAP, 4) = base * (base * (base * base)) */
  }
  g->pot = pot;
  g->NEcharge = Ncharge * Echarge;
  g->EEcharge = Echarge * Echarge;
  g->Nsoft = Nsoft;
  g->Esoft = Esoft;
  g->gauge = gauge;
  g->n_fields = n_fields;
  g->p_swap = dim >= 2 ? 1 : 0;
}

/* Region `free_mask` of a multi-region grid (mpi_logic.h:104-150, multigrid.h:11-47):
 * only the main region (free_mask 0) keeps the transposed P layout
 * (canLeaveTransposed, grid.h:118) */
void orc_grid_set_region(orc_grid* g, int free_mask, int multi) {
  g->free_mask = free_mask;
  g->multi = multi;
  g->p_swap = (g->dim >= 2 && free_mask == 0) ? 1 : 0;
}

/* The cos^(1/8) mask absorber of the 1D plain configuration's text (no reference
 * counterpart: the reference has only the quartic CAP of absorbers.h).  Over the same
 * margin of nCAP nodes per side, node depth nodes = nCAP + neg_dist_from_edge (nCAP at
 * the outermost node, 1 at the innermost margin node), the mask of one axis is
 * M_d = cos(pi/2 * nodes / nCAP)^(1/8) and of a point the product over axes.  It is
 * applied once per mask_dt of propagation: evolve<X>(delta) multiplies by
 * M^(delta / mask_dt), so the two X halves of a Strang step of dt = mask_dt apply M once. */
void orc_grid_set_absorber(orc_grid* g, int kind, double mask_dt) {
  g->abs_kind = kind;
  g->abs_rate = (kind == 1 && mask_dt > 0.0) ? 1.0 / mask_dt : 0.0;
}

/* coords.h:132-138 */
static inline double pos(const orc_grid* g, int rep, int d, long i) {
  if (rep == ORC_REP_X) return g->xmin[d] + (double)i * g->dx[d];
  return g->dp[d] * (double)(i < g->n2[d] ? i : i - g->n[d]);
}

/* potential.h:130-143 (ReducedDimInteraction), potential.h:40-44 (CoulombInteraction) */
static inline double ee_i(const orc_grid* g, double x, double y) {
  if (g->pot == ORC_POT_ECKHARDT_SACHA) return g->EEcharge / sqrt((x - y) * (x - y) + x * y + g->Esoft);
  return g->EEcharge / sqrt((x - y) * (x - y) + g->Esoft);
}
static inline double Ne_i(const orc_grid* g, double x) { return g->NEcharge / sqrt(x * x + g->Nsoft); }

/* ReducedDimInteraction::partial (potential.h:144-178): interactions of the bounded
 * coordinates only; fc = free-axis mask (1 X, 2 Y, 4 Z) */
static inline double partial_potential(const orc_grid* g, int fc, const double* c) {
  if (g->dim == 1) return fc == 0 ? Ne_i(g, c[0]) : 0.0;
  if (g->dim == 2) {
    if (fc == 0) return ee_i(g, c[0], c[1]) + Ne_i(g, c[0]) + Ne_i(g, c[1]);
    if (fc == 2) return Ne_i(g, c[0]);
    if (fc == 1) return Ne_i(g, c[1]);
    return 0.0;
  }
  switch (fc) {
    case 0: return ee_i(g, c[0], c[1]) + ee_i(g, c[1], c[2]) + ee_i(g, c[2], c[0]) + Ne_i(g, c[0]) + Ne_i(g, c[1]) +
                   Ne_i(g, c[2]);
    case 4: return ee_i(g, c[0], c[1]) + Ne_i(g, c[0]) + Ne_i(g, c[1]);
    case 2: return ee_i(g, c[0], c[2]) + Ne_i(g, c[0]) + Ne_i(g, c[2]);
    case 1: return ee_i(g, c[1], c[2]) + Ne_i(g, c[1]) + Ne_i(g, c[2]);
    case 6: return Ne_i(g, c[0]);
    case 5: return Ne_i(g, c[1]);
    case 3: return Ne_i(g, c[2]);
    default: return 0.0;
  }
}

static inline double potential(const orc_grid* g, const double* c) {
  if (g->pot == ORC_POT_NONE) return 0.0;
  if (g->multi) return partial_potential(g, g->free_mask, c);
  if (g->pot == ORC_POT_COULOMB) {
    double s;
    if (g->dim == 1) s = c[0] * c[0];
    else if (g->dim == 2) s = c[0] * c[0] + c[1] * c[1];
    else s = c[0] * c[0] + (c[1] * c[1] + c[2] * c[2]);
    return g->NEcharge / sqrt(s + g->Nsoft);
  }
  if (g->dim == 1) return Ne_i(g, c[0]);
  if (g->dim == 2) return ee_i(g, c[0], c[1]) + Ne_i(g, c[0]) + Ne_i(g, c[1]);
  return ee_i(g, c[0], c[1]) + ee_i(g, c[1], c[2]) + ee_i(g, c[2], c[0]) + Ne_i(g, c[0]) +
         Ne_i(g, c[1]) + Ne_i(g, c[2]);
}

/* hamiltonian.h:44-58 (coupling, kinetic); folds ((a) + ...) are right folds */
static inline double kinetic(const orc_grid* g, const double* k) {
  if (g->dim == 1) return 0.5 * k[0] * k[0];
  if (g->dim == 2) return 0.5 * k[0] * k[0] + 0.5 * k[1] * k[1];
  return 0.5 * k[0] * k[0] + (0.5 * k[1] * k[1] + 0.5 * k[2] * k[2]);
}
static inline double coupling_term(const orc_grid* g, int rep, const double* c, const double* cv) {
  int couples = g->gauge == ORC_GAUGE_VELOCITY ? ORC_REP_P : ORC_REP_X;
  if (couples != rep || g->n_fields == 0 || cv == NULL) return 0.0;
  if (g->dim == 1) return c[0] * cv[0];
  if (g->dim == 2) return c[0] * cv[0] + c[1] * cv[1];
  return c[0] * cv[0] + (c[1] * cv[1] + c[2] * cv[2]);
}

/* grid.h:181-185 */
static inline long neg_dist_from_edge(const orc_grid* g, int d, long i) {
  return i < g->n2[d] ? -i : i - g->n[d] + 1;
}

/* absorbers.h:40-46 */
static inline double absorb(const orc_grid* g, double delta, const long* nodes_in) {
  long nodes[3];
  int all_neg = 1;
  for (int d = 0; d < g->dim; ++d) {
    nodes[d] = g->nCAP + nodes_in[d];
    if (!(nodes[d] < 0)) all_neg = 0;
  }
  if (all_neg) return 1.0;
  if (g->abs_kind == 1) { /* cos^(1/8) mask to the power delta / mask_dt */
    double lsum = 0.0;
    for (int d = 0; d < g->dim; ++d)
      if (nodes[d] > 0) lsum += log(cos(1.5707963267948966 * ((double)nodes[d] / (double)g->nCAP)));
    return exp(delta * g->abs_rate * 0.125 * lsum);
  }
  long s = 0;
  for (int d = g->dim - 1; d >= 0; --d) {
    long v = nodes[d] > 0 ? nodes[d] * (nodes[d] * (nodes[d] * nodes[d])) : 0;
    s = v + s;
  }
  return exp(-delta * (double)s * g->eta);
}

/* absorbers.h:48-54 (mask), grid.h:582-597 (maskRegion_): bounded[d]==0 -> -n2 */
double orc_mask_value(const orc_grid* g, const long* idx, const int* bounded) {
  long nodes[3];
  int all_neg = 1;
  for (int d = 0; d < g->dim; ++d) {
    long nd = bounded[d] ? neg_dist_from_edge(g, d, idx[d]) : -g->n2[d];
    nodes[d] = g->nCAP + nd;
    if (!(nodes[d] < 0)) all_neg = 0;
  }
  if (all_neg) return 1.0;
  long s = 0;
  for (int d = g->dim - 1; d >= 0; --d) {
    long v = nodes[d] > 0 ? nodes[d] * (nodes[d] * (nodes[d] * nodes[d])) : 0;
    s = v + s;
  }
  return exp(-(double)(s + 0) * g->eta);
}

void orc_mask_region(const orc_grid* g, double* psi_d, const int* bounded) {
  orc_cx* psi = (orc_cx*)psi_d;
  long idx[3] = {0, 0, 0};
  for (long c = 0; c < g->m; ++c) {
    long r = c;
    for (int d = g->dim - 1; d >= 0; --d) { idx[d] = r % g->n[d]; r /= g->n[d]; }
    double mk = orc_mask_value(g, idx, bounded);
    psi[c].re *= mk;
    psi[c].im *= mk;
  }
}

/* CAP::mask of one node (absorbers.h:48-54): 1 outside the margin */
static inline double mask1(const orc_grid* g, long nd) {
  long nodes = g->nCAP + nd;
  if (nodes < 0) return 1.0;
  double v = nodes > 0 ? (double)(nodes * (nodes * (nodes * nodes))) : 0.0;
  return exp(-(v + 0) * g->eta);
}

/* Region transfer (multigrid.h:454-615, one source): the absorber margins of `src`
 * along axis fc (both edges; in 3D only the boxes of nCAP planes along the sliding
 * axis, n / nCAP of them) times inv_mask(fc) and, for a destination in group 1, the
 * corner correction; then the forward DFT along fc (unnormalised) and dst += slice.
 * In 1D getBox copies whole rows, and the one row is the whole line: the interior
 * between the margins enters the slice unmasked (getBox / maskSlice, multigrid.h:
 * 454-481, 532-569, with an empty index pack). */
void orc_mg_transfer(const orc_grid* g, double* dst_d, const double* src_d, int fc, int group) {
  const orc_cx* src = (const orc_cx*)src_d;
  orc_cx* dst = (orc_cx*)dst_d;
  orc_cx* slice = (orc_cx*)calloc((size_t)g->m, sizeof(orc_cx));
  const int D = g->dim;
  const int slide = D == 3 ? (fc == 1 ? 2 : 1) : -1;
  const long slide_lim = D == 3 ? (g->n[0] / g->nCAP) * g->nCAP : 0;
  long idx[3] = {0, 0, 0};
  for (long p = 0; p < g->m; ++p) {
    long r = p;
    for (int d = D - 1; d >= 0; --d) { idx[d] = r % g->n[d]; r /= g->n[d]; }
    const long i = idx[fc];
    if (!(i < g->nCAP || i >= g->n[fc] - g->nCAP)) {
      if (D == 1) slice[p] = src[p];
      continue;
    }
    if (slide >= 0 && idx[slide] >= slide_lim) continue;
    const double mv = 1.0 - mask1(g, neg_dist_from_edge(g, fc, i));
    double f = mv;
    if (group == 1) {
      double corr = 1.0;
      if (D == 2) {
        const int o = 1 - fc;
        const double b0 = fc == 0 ? 1.0 : 1.0 - mask1(g, neg_dist_from_edge(g, o, idx[o]));
        const double b1 = fc == 1 ? 1.0 : 1.0 - mask1(g, neg_dist_from_edge(g, o, idx[o]));
        corr = 1 - 0.5 * (b0 * b1);
      } else if (D == 3) {
        double a[3], b[3];
        for (int d = 0; d < 3; ++d) {
          const double mk = mask1(g, neg_dist_from_edge(g, d, idx[d]));
          a[d] = d == fc ? 0 : mk;
          b[d] = d == fc ? 1.0 : mk;
        }
        corr = 0.5 * (a[0] + (a[1] + (a[2] + 0))) + (1.0 / 6.0) * (1 - (b[0] * (b[1] * b[2])));
      }
      f = mv * corr;
    }
    slice[p].re = src[p].re * f;
    slice[p].im = src[p].im * f;
  }
  int use[3] = {0, 0, 0};
  use[fc] = 1;
  orc_fft_axes((double*)slice, D, g->n, use, -1);
  for (long p = 0; p < g->m; ++p) {
    dst[p].re += slice[p].re;
    dst[p].im += slice[p].im;
  }
  free(slice);
}

/* coupling vector as seen by the P-space loop; the reference's P layout for dim>1 is
 * axis-0/1 transposed (grid.h:242-247), so its loop applies the axis-0 coupling to
 * the physical axis-1 wavenumber; on square grids this equals a swap of cv[0], cv[1]. */
static inline void p_coupling(const orc_grid* g, const double* cv, double* out) {
  for (int d = 0; d < 3; ++d) out[d] = cv ? cv[d] : 0.0;
  if (g->p_swap && g->dim >= 2 && cv) { out[0] = cv[1]; out[1] = cv[0]; }
}

/* grid.h:394-418 (evolve_), hamiltonian.h:73-79 (operator()), 92-97 (expOp) */
void orc_evolve(const orc_grid* g, double* psi_d, int mode, int rep, double delta, const double* cv_in) {
  orc_cx* psi = (orc_cx*)psi_d;
  double cv[3];
  if (rep == ORC_REP_P) p_coupling(g, cv_in, cv);
  else for (int d = 0; d < 3; ++d) cv[d] = cv_in ? cv_in[d] : 0.0;
  long idx[3] = {0, 0, 0};
  double c[3];
  long nodes[3];
  for (long i = 0; i < g->m; ++i) {
    long r = i;
    for (int d = g->dim - 1; d >= 0; --d) { idx[d] = r % g->n[d]; r /= g->n[d]; }
    for (int d = 0; d < g->dim; ++d) c[d] = pos(g, rep, d, idx[d]);
    double H;
    if (rep == ORC_REP_P) H = kinetic(g, c) + coupling_term(g, rep, c, cv);
    else H = potential(g, c) + coupling_term(g, rep, c, cv);
    double val = delta * H;
    if (mode == ORC_MODE_IM) {
      double f = exp(-val);
      psi[i].re *= f;
      psi[i].im *= f;
    } else {
      orc_cx f = {cos(-val), sin(-val)};
      psi[i] = cmul(psi[i], f);
    }
    if (rep == ORC_REP_X && g->nCAP > 0 && !g->multi) {
      for (int d = 0; d < g->dim; ++d) nodes[d] = neg_dist_from_edge(g, d, idx[d]);
      double a = absorb(g, delta, nodes);
      psi[i].re *= a;
      psi[i].im *= a;
    }
  }
}

/* grid.h:369-378 (fourier) + 363-367 (normalizeAfterTwoFFT) */
void orc_fourier(const orc_grid* g, double* psi_d, int to_rep) {
  if (g->free_mask) {
    /* fourier_partial (multigrid.h:660-674): the bounded axes only, then the product of
     * their 1/n on the way back (when there is any bounded axis) */
    int use[3] = {0, 0, 0}, any = 0;
    double s = 1.0;
    for (int d = 0; d < g->dim; ++d) {
      use[d] = !((g->free_mask >> d) & 1);
      any |= use[d];
      s *= use[d] ? 1.0 / (double)g->n[d] : 1.0;
    }
    if (!any) return;
    orc_fft_axes(psi_d, g->dim, g->n, use, to_rep == ORC_REP_P ? -1 : +1);
    if (to_rep == ORC_REP_X) {
      orc_cx* psi = (orc_cx*)psi_d;
      for (long i = 0; i < g->m; ++i) { psi[i].re *= s; psi[i].im *= s; }
    }
    return;
  }
  orc_fft_nd(psi_d, g->dim, g->n, to_rep == ORC_REP_P ? -1 : +1);
  if (to_rep == ORC_REP_X) {
    orc_cx* psi = (orc_cx*)psi_d;
    for (long i = 0; i < g->m; ++i) { psi[i].re *= g->inv_m; psi[i].im *= g->inv_m; }
  }
}

/* grid.h:425-441 (average_), hamiltonian.h:81-90 (call), coords.h:27-32 (vol) */
double orc_average(const orc_grid* g, const double* psi_d, int rep, int op) {
  const orc_cx* psi = (const orc_cx*)psi_d;
  long idx[3] = {0, 0, 0};
  double c[3];
  double res = 0.0;
  for (long i = 0; i < g->m; ++i) {
    double w = 1.0;
    if (op != ORC_OP_IDENTITY) {
      long r = i;
      for (int d = g->dim - 1; d >= 0; --d) { idx[d] = r % g->n[d]; r /= g->n[d]; }
      if (op == ORC_OP_KINETIC) {
        for (int d = 0; d < g->dim; ++d) c[d] = pos(g, rep, d, idx[d]);
        w = kinetic(g, c);
      } else {
        for (int d = 0; d < g->dim; ++d) c[d] = pos(g, rep, d, idx[d]);
        w = potential(g, c);
      }
    }
    res += (psi[i].re * psi[i].re + psi[i].im * psi[i].im) * w;
  }
  return res * (rep == ORC_REP_X ? g->dV : g->dVm);
}

/* average_der_<X, dir, Op> (grid.h:443-465) with Op = PotentialEnergy (hamiltonian.h:81-90):
 * sum_i |psi_i|^2 (V(x_i + dx e_dir) - V(x_i - dx e_dir)) dV / (2 dx_dir), positions one
 * node past either edge taken from the same linear formula (coords.h:132-135) */
double orc_average_der(const orc_grid* g, const double* psi_d, int dir) {
  const orc_cx* psi = (const orc_cx*)psi_d;
  long idx[3] = {0, 0, 0};
  double cp[3], cm[3];
  double res = 0.0;
  for (long i = 0; i < g->m; ++i) {
    long r = i;
    for (int d = g->dim - 1; d >= 0; --d) { idx[d] = r % g->n[d]; r /= g->n[d]; }
    for (int d = 0; d < g->dim; ++d) {
      cp[d] = pos(g, ORC_REP_X, d, idx[d] + (d == dir ? 1 : 0));
      cm[d] = pos(g, ORC_REP_X, d, idx[d] + (d == dir ? -1 : 0));
    }
    res += (psi[i].re * psi[i].re + psi[i].im * psi[i].im) * (potential(g, cp) - potential(g, cm));
  }
  return res * g->dV * g->inv_2dx[dir];
}

/* operation<M, R, AntiSymmetrize<particles>> on one rank (grid.h:611-723).
 * particles 2, dim 2: psi(i,j) -= psi_copy(j,i).
 * particles 2, dim 3 (partial, axes 1 and 2): for k < j: psi(i,j,k) -= psi(i,k,j),
 *   psi(i,k,j) = -psi(i,j,k); psi(i,j,j) = 0.
 * particles 3, dim 3: for i > j > k the even permutations get
 *   psi(i,j,k) + psi(j,k,i) + psi(k,i,j) - psi(j,i,k) - psi(i,k,j) - psi(k,j,i), the odd
 *   ones its negative; every point with two equal indices becomes 0.
 * Other (particles, dim) combinations leave psi unchanged, as the reference does. */
void orc_antisymmetrize(const orc_grid* g, double* psi_d, int particles) {
  orc_cx* psi = (orc_cx*)psi_d;
  const long n = g->n[0];
  if (particles == 2 && g->dim == 2) {
    orc_cx* copy = (orc_cx*)malloc(sizeof(orc_cx) * (size_t)g->m);
    memcpy(copy, psi, sizeof(orc_cx) * (size_t)g->m);
    for (long i = 0; i < n; ++i)
      for (long j = 0; j < n; ++j) {
        psi[i * n + j].re -= copy[j * n + i].re;
        psi[i * n + j].im -= copy[j * n + i].im;
      }
    free(copy);
  } else if (particles == 2 && g->dim == 3) {
    for (long i = 0; i < n; ++i)
      for (long j = 0; j < n; ++j) {
        for (long k = 0; k < j; ++k) {
          orc_cx* a = &psi[(i * n + j) * n + k];
          orc_cx* b = &psi[(i * n + k) * n + j];
          a->re -= b->re;
          a->im -= b->im;
          b->re = -a->re;
          b->im = -a->im;
        }
        psi[(i * n + j) * n + j].re = 0.0;
        psi[(i * n + j) * n + j].im = 0.0;
      }
  } else if (particles == 3 && g->dim == 3) {
#define AT(a, b, c) psi[((a) * n + (b)) * n + (c)]
    for (long i = 0; i < n; ++i) {
      for (long j = 0; j < i; ++j)
        for (long k = 0; k < j; ++k) {
          orc_cx s;
          s.re = AT(j, k, i).re + AT(k, i, j).re - AT(j, i, k).re - AT(i, k, j).re - AT(k, j, i).re;
          s.im = AT(j, k, i).im + AT(k, i, j).im - AT(j, i, k).im - AT(i, k, j).im - AT(k, j, i).im;
          AT(i, j, k).re += s.re;
          AT(i, j, k).im += s.im;
          const orc_cx v = AT(i, j, k);
          AT(j, k, i) = v;
          AT(k, i, j) = v;
          AT(j, i, k).re = -v.re; AT(j, i, k).im = -v.im;
          AT(i, k, j).re = -v.re; AT(i, k, j).im = -v.im;
          AT(k, j, i).re = -v.re; AT(k, j, i).im = -v.im;
        }
      for (long j = 0; j < n; ++j) {
        AT(i, j, j).re = AT(i, j, j).im = 0.0;
        AT(j, i, j).re = AT(j, i, j).im = 0.0;
        AT(j, j, i).re = AT(j, j, i).im = 0.0;
      }
    }
#undef AT
  }
}

/* grid.h:601-606 (operation<Normalize>); returns the norm it divided by */
double orc_normalize(const orc_grid* g, double* psi_d) {
  double res = orc_average(g, psi_d, ORC_REP_X, ORC_OP_IDENTITY);
  double s = sqrt(1.0 / res);
  orc_cx* psi = (orc_cx*)psi_d;
  for (long i = 0; i < g->m; ++i) { psi[i].re *= s; psi[i].im *= s; }
  return res;
}

/* grid.h:467-528 (update_curr, current_map_) + propagator.h:249-257 (velocity-gauge
 * correction).  curr has dim doubles per point. */
void orc_current_map(const orc_grid* g, const double* psi_d, const double* A_vg, double* curr) {
  const orc_cx* psi = (const orc_cx*)psi_d;
  for (long c = 0; c < g->m; ++c) {
    for (int d = 0; d < g->dim; ++d) {
      long s = g->stride[d];
      double v = 0.0;
      if ((c - s > 0) && (c + s < g->m)) {
        orc_cx t = {psi[c + s].re - psi[c - s].re, psi[c + s].im - psi[c - s].im};
        /* imag(conj(psi) * t) */
        v = g->inv_2dx[d] * (psi[c].re * t.im + (-psi[c].im) * t.re);
      }
      curr[c * g->dim + d] = v;
    }
  }
  if (A_vg) {
    for (long c = 0; c < g->m; ++c) {
      double nrm = psi[c].re * psi[c].re + psi[c].im * psi[c].im;
      for (int d = 0; d < g->dim; ++d) curr[c * g->dim + d] += A_vg[d] * nrm;
    }
  }
}

/* ---------------------------------------------------------- flux borders */
/* fluxes/borders_g.h:1-40, borders_t.h:1-13, borders.h:30-257 */

static long g_p_NS = 25, g_p_SD = 14, g_p_DT = 10, g_p_CAP = 40;

void orc_set_border_nodes(long p_NS, long p_SD, long p_DT, long p_CAP) {
  g_p_NS = p_NS; g_p_SD = p_SD; g_p_DT = p_DT; g_p_CAP = p_CAP;
}

static inline double Sign(long x) { return (double)((x > 0) - (x < 0)); }
static inline int Rn(long i, long il, long ir) { return i >= il && i < ir; }
static inline int Rn2(long i, long il, long ir) { return Rn(i, il, ir) || Rn(i, -ir, -il); }
static inline double PointB(long i, long iat) { return i == iat - 1 ? Sign(i) : 0; }
static inline double PointB2(long i, long iat) { return (i == iat - 1 || i == -iat) ? Sign(i) : 0; }
static inline double SegmentB(long i, long j, long jat, long il, long ir) { return Rn(i, il, ir) ? PointB(j, jat) : 0; }
static inline double SegmentBi2j2(long i, long j, long jat, long il, long ir) { return Rn2(i, il, ir) ? PointB2(j, jat) : 0; }
static inline double SegmentBi2(long i, long j, long jat, long il, long ir) { return Rn2(i, il, ir) ? PointB(j, jat) : 0; }
static inline double PatchBi2j2k2(long i, long j, long k, long kat, long il, long ir, long jl, long jr) {
  return Rn2(i, il, ir) ? (Rn2(j, jl, jr) ? PointB2(k, kat) : 0) : 0;
}

/* borVec normalisation (borders_t.h:6-13) */
static void bor_norm(double* v, int dim) {
  double s = 0.0;
  for (int d = 0; d < dim; ++d) s = s + v[d] * v[d];
  double nrm = sqrt(s + 0.0);
  if (nrm > 0.001)
    for (int d = 0; d < dim; ++d) v[d] /= nrm;
}

enum {
  ORC_B_BOX = 0, ORC_B_S2CAP, ORC_B_D2CAP, ORC_B_N2S, ORC_B_N2D, ORC_B_N2D_SYM, ORC_B_N2D_ASYM,
  ORC_B_S2D, ORC_B_S2D_SYM, ORC_B_S2D_ASYM, ORC_B_N2T, ORC_B_S2T, ORC_B_D2T, ORC_B_T2CAP
};

/* Outward border vector of type `type` at centred indices (i[, j[, k]]). */
void orc_border(int type, long box_size, int dim, const long* ci, double* out) {
  long i = ci[0], j = dim > 1 ? ci[1] : 0, k = dim > 2 ? ci[2] : 0;
  long NS = g_p_NS, SD = g_p_SD, DT = g_p_DT, CAP = g_p_CAP;
  for (int d = 0; d < 3; ++d) out[d] = 0.0;
#define P3(a, b, c, kat, il, ir, jl, jr) PatchBi2j2k2(a, b, c, kat, il, ir, jl, jr)
#define SYM3(kat, il, ir, jl, jr)                                                   \
  out[0] = P3(j, k, i, kat, il, ir, jl, jr) + P3(k, j, i, kat, il, ir, jl, jr);       \
  out[1] = P3(k, i, j, kat, il, ir, jl, jr) + P3(i, k, j, kat, il, ir, jl, jr);       \
  out[2] = P3(i, j, k, kat, il, ir, jl, jr) + P3(j, i, k, kat, il, ir, jl, jr);
#define PLAIN3(kat, il, ir, jl, jr)          \
  out[0] = P3(j, k, i, kat, il, ir, jl, jr); \
  out[1] = P3(k, i, j, kat, il, ir, jl, jr); \
  out[2] = P3(i, j, k, kat, il, ir, jl, jr);
  switch (type) {
    case ORC_B_BOX:
      if (dim == 1) out[0] = PointB2(i, box_size);
      else if (dim == 2) {
        out[0] = SegmentBi2j2(j, i, box_size, 0, box_size);
        out[1] = SegmentBi2j2(i, j, box_size, 0, box_size);
      } else { PLAIN3(box_size, 0, box_size, 0, box_size) }
      break;
    case ORC_B_S2CAP:
      if (dim == 2) { out[0] = SegmentBi2j2(j, i, CAP, 0, SD); out[1] = SegmentBi2j2(i, j, CAP, 0, SD); }
      else { SYM3(CAP, 0, DT, 0, SD) }
      break;
    case ORC_B_D2CAP:
      if (dim == 2) { out[0] = SegmentBi2j2(j, i, CAP, SD, CAP); out[1] = SegmentBi2j2(i, j, CAP, SD, CAP); }
      else { SYM3(CAP, SD, CAP, 0, DT) }
      break;
    case ORC_B_N2S:
      if (dim == 2) { out[0] = SegmentBi2j2(j, i, NS, 0, SD); out[1] = SegmentBi2j2(i, j, NS, 0, SD); }
      else { SYM3(NS, 0, SD, 0, DT - 1) }
      break;
    case ORC_B_N2D:
      if (dim == 2) { out[0] = SegmentBi2j2(j, i, SD, SD, NS); out[1] = SegmentBi2j2(i, j, SD, SD, NS); }
      else { SYM3(SD, SD, NS, 0, DT - 1) }
      break;
    case ORC_B_N2D_SYM:
      out[0] = SegmentB(j + 1, i, SD, SD, NS + 1) - SegmentB(-j, -i - 1, SD, SD, NS + 1);
      out[1] = SegmentB(i + 1, j, SD, SD, NS + 1) - SegmentB(-i, -j - 1, SD, SD, NS + 1);
      break;
    case ORC_B_N2D_ASYM:
      out[0] = -SegmentB(j + 1, -i - 1, SD, SD, NS + 1) + SegmentB(-j, i, SD, SD, NS + 1);
      out[1] = -SegmentB(i + 1, -j - 1, SD, SD, NS + 1) + SegmentB(-i, j, SD, SD, NS + 1);
      break;
    case ORC_B_S2D:
      if (dim == 2) { out[0] = SegmentBi2j2(j, i, SD, NS, CAP); out[1] = SegmentBi2j2(i, j, SD, NS, CAP); }
      else { SYM3(SD, NS, CAP, 0, DT) }
      break;
    case ORC_B_S2D_SYM:
      out[0] = SegmentB(j, i, SD, NS, CAP) - SegmentB(-j - 1, -i - 1, SD, NS, CAP);
      out[1] = SegmentB(i, j, SD, NS, CAP) - SegmentB(-i - 1, -j - 1, SD, NS, CAP);
      break;
    case ORC_B_S2D_ASYM:
      out[0] = -SegmentB(j, -i - 1, SD, NS, CAP) + SegmentB(-j - 1, i, SD, NS, CAP);
      out[1] = -SegmentB(i, -j - 1, SD, NS, CAP) + SegmentB(-i - 1, j, SD, NS, CAP);
      break;
    case ORC_B_N2T: SYM3(DT, DT - 1, NS, DT - 1, SD) break;
    case ORC_B_S2T: SYM3(DT, NS, CAP, DT, SD) break;
    case ORC_B_D2T: PLAIN3(DT, SD, CAP, SD, CAP) break;
    case ORC_B_T2CAP: PLAIN3(CAP, DT, CAP, DT, CAP) break;
    default: break;
  }
#undef P3
#undef SYM3
#undef PLAIN3
  bor_norm(out, dim);
}

/* grid.h:559-573 (flux_): sum_i curr[i] . border(centred index) * dV / dx[0] */
double orc_flux(const orc_grid* g, const double* curr, int type, long box_size) {
  long idx[3] = {0, 0, 0}, ci[3];
  double b[3];
  double res = 0.0;
  for (long c = 0; c < g->m; ++c) {
    long r = c;
    for (int d = g->dim - 1; d >= 0; --d) { idx[d] = r % g->n[d]; r /= g->n[d]; }
    for (int d = 0; d < g->dim; ++d) ci[d] = idx[d] - g->n2[d];
    orc_border(type, box_size, g->dim, ci, b);
    double dot = 0.0;
    for (int d = 0; d < g->dim; ++d) dot += curr[c * g->dim + d] * b[d];
    res += dot;
  }
  return res * g->dV / g->dx[0];
}

/* ------------------------------------------------------------ fields */
/* field_p.h:6-12 (_FieldConfig), 30-33 (PulsePrototype), 47-56 (SinPulse),
 * 67-78 (ChemPhysPulse), 100-116 (Sin2Envelope), field.h:23-37 (Field::operator()),
 * field.h:114-123 (PromoteFieldToA). */
enum { ORC_PULSE_SIN = 0, ORC_PULSE_SIN2_SIN = 1, ORC_PULSE_CONST = 2, ORC_PULSE_CHEMPHYS = 3 };

typedef struct {
  int shape;
  double field, omega, ncycles, FWHM_percent, phase_in_pi_units, delay_in_cycles;
} orc_pulse;

static double pulse_eval(const orc_pulse* p, double time) {
  double phi = p->phase_in_pi_units * M_PI;
  switch (p->shape) {
    case ORC_PULSE_SIN: return p->field * sin(p->omega * time + phi);
    case ORC_PULSE_SIN2_SIN: {
      double env_mult = p->omega / (2.0 * p->ncycles);
      double s = sin(env_mult * time);
      return p->field * sin(p->omega * time + phi) * (s * s);
    }
    case ORC_PULSE_CONST: return p->field;
    case ORC_PULSE_CHEMPHYS: {
      double env_mult = p->omega / (2.0 * p->ncycles);
      double tmp = p->omega * time + phi - M_PI * p->ncycles;
      return p->field * (sin(env_mult * time) * cos(tmp) + cos(env_mult * time) * sin(tmp) / p->ncycles);
    }
  }
  return 0.0;
}

/* Field<Ax, Pulses...>::operator()(time): sum of active pulses */
double orc_field_eval(const orc_pulse* pulses, int npulses, double time) {
  double val = 0.0;
  for (int i = 0; i < npulses; ++i) {
    const orc_pulse* p = &pulses[i];
    double delay = p->delay_in_cycles * 2.0 * M_PI / p->omega;
    double endt = delay + 2.0 * M_PI * p->ncycles / p->omega;
    val += (!(time > endt || time < delay)) ? pulse_eval(p, time - delay) : 0.0;
  }
  return val;
}

double orc_field_max_duration(const orc_pulse* pulses, int npulses) {
  double mx = 0.0;
  for (int i = 0; i < npulses; ++i) {
    const orc_pulse* p = &pulses[i];
    double endt = p->delay_in_cycles * 2.0 * M_PI / p->omega + 2.0 * M_PI * p->ncycles / p->omega;
    if (i == 0 || mx < endt) mx = endt;
  }
  return mx;
}

/* PromoteFieldToA state: A_n = A_{n-1} + (t_{n-1} - t_n) F(t_n) */
typedef struct { double lastVal, prevTime; } orc_astate;

double orc_vector_potential_step(orc_astate* s, const orc_pulse* pulses, int npulses, double time) {
  double prev = s->lastVal;
  double F = orc_field_eval(pulses, npulses, time);
  s->lastVal = prev + (s->prevTime - time) * F;
  s->prevTime = time;
  return s->lastVal;
}

/* ------------------------------------------------------------- helpers */

/* wf/preset.h:5-10 gaussian(at, delta, coords...) filled via addUsingCoordinateFunction
 * (grid.h:775-778, add<F,R,true>: psi += f(x...)) */
void orc_add_gaussian(const orc_grid* g, double* psi_d, double at, double delta) {
  orc_cx* psi = (orc_cx*)psi_d;
  long idx[3];
  double delta_inv = 1.0 / delta;
  double base = sqrt(delta_inv * sqrt(1.0 / M_PI));
  double nrm = 1.0;
  /* Power(base, dim) */
  if (g->dim == 1) nrm = base;
  else if (g->dim == 2) nrm = base * base;
  else nrm = base * (base * base);
  for (long c = 0; c < g->m; ++c) {
    long r = c;
    for (int d = g->dim - 1; d >= 0; --d) { idx[d] = r % g->n[d]; r /= g->n[d]; }
    double x[3];
    for (int d = 0; d < g->dim; ++d) x[d] = pos(g, ORC_REP_X, d, idx[d]);
    double s;
    if (g->dim == 1) s = (x[0] - at) * (x[0] - at) * delta_inv * delta_inv;
    else if (g->dim == 2)
      s = (x[0] - at) * (x[0] - at) * delta_inv * delta_inv + (x[1] - at) * (x[1] - at) * delta_inv * delta_inv;
    else
      s = (x[0] - at) * (x[0] - at) * delta_inv * delta_inv +
          ((x[1] - at) * (x[1] - at) * delta_inv * delta_inv + (x[2] - at) * (x[2] - at) * delta_inv * delta_inv);
    psi[c].re += exp(-0.5 * s) * nrm;
  }
}

/* sizeof helper for the ctypes wrapper */
int orc_sizeof_grid(void) { return (int)sizeof(orc_grid); }
