/*
 * tree2d_sparse.c -- sparse restatement of the reference tree, and an
 * extended-precision evaluation of the same treecode.
 *
 * TEST INFRASTRUCTURE ONLY (compiled into liboracle.so beside
 * tree2d_oracle.c).  Nothing in the product library links, loads or calls
 * this file.
 *
 * 1. Sparse tree.  tree2d_oracle.c keeps the reference's dense complete
 *    quadtree of (4^(L+1)-1)/3 nodes, which cannot be allocated past about
 *    15 levels.  Here the same tree is built with only the nodes the
 *    reference ever creates (every child of every split cell, empty ones
 *    included), by the same rules in the same order:
 *      - root box ............ ver-c/src/quadtree.c:81-99   (calc_region)
 *      - quadrant test ....... ver-c/src/quadtree.c:29-35   (quadrant_pos)
 *      - child centres ....... ver-c/src/quadtree.c:61-79   (calc_CenterPos)
 *      - LIFO splitting ...... ver-c/src/quadtree.c:173-251 (split_cell):
 *        children keep the parent's order, a child with >= num_p blobs is
 *        pushed, the stack pops last-pushed first;
 *      - S2M / M2M ........... ver-c/src/fmm.c:18-58: the reference runs
 *        M2M over node ids in descending order, so every level is finished
 *        before the level above reads it, and each parent adds its children
 *        3, 2, 1, 0 in that order; the level-1 -> root shift is not done.
 *        Here: deepest level first, children 3..0 per parent, the same sums;
 *      - biot_tree ........... ver-c/src/fmm.c:69-118: LIFO from the root,
 *        children 0..3 tested region > theta*r, push or M2S; leaves P2P.
 *    The reference's max-level retry loop (quadtree.c:102-171) changes only
 *    its allocation, not the tree, so the sparse build splits until every
 *    leaf holds < num_p blobs (up to a level cap for coincident blobs).
 *    The floating-point expressions are the reference's, as in
 *    tree2d_oracle.c, and the tests hold this tree bit-exact against the
 *    dense one on every golden case.
 *
 * 2. Extended precision.  ora_sp_biot_ext evaluates the same treecode --
 *    the same accepted cells and the same direct pairs, decided in FP64 as
 *    the reference decides them -- with every coefficient (S2M, M2M) and
 *    every M2S and P2P term in long double (64-bit significand on x86-64,
 *    113-bit on AArch64) and powers by repeated multiplication instead of
 *    cpow.  Its result is the treecode's value to far below FP64 rounding,
 *    so |reference - ext| is the reference's own rounding (cpow = exp(k log
 *    z) carries error growing with k |log z|) and |gpu - ext| the GPU's.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* parameters in force (set through ora_set_params in tree2d_oracle.c) */
int ora_nterms(void);
int ora_num_p(void);
double ora_theta(void);

typedef long double complex ldc;

typedef struct {
  int level;
  int nb;
  int *ids;          /* blob ids in bucketing order                  */
  double c[2];
  double region;
  int leaf;
  long child[4];     /* -1 until split                               */
  double complex *a; /* FP64 coefficients (the reference's)          */
  ldc *ae;           /* extended-precision coefficients (on demand)  */
} sp_node;

static struct {
  int nterms, num_p;
  double theta;
  int levels;
  long nn, cap;
  sp_node *node;
  double *x, *y, *cir, *cor;
  int n;
  int have_ext;
} S;

static void sp_free(void) {
  for (long i = 0; i < S.nn; i++) {
    free(S.node[i].ids);
    free(S.node[i].a);
    free(S.node[i].ae);
  }
  free(S.node);
  free(S.x);
  free(S.y);
  free(S.cir);
  free(S.cor);
  memset(&S, 0, sizeof(S));
}

static long sp_new(int level) {
  if (S.nn == S.cap) {
    S.cap = S.cap ? 2 * S.cap : 1024;
    S.node = (sp_node *)realloc(S.node, sizeof(sp_node) * (size_t)S.cap);
  }
  sp_node *nd = &S.node[S.nn];
  memset(nd, 0, sizeof(*nd));
  nd->level = level;
  for (int q = 0; q < 4; q++) nd->child[q] = -1;
  nd->a = (double complex *)calloc((size_t)(S.nterms > 0 ? S.nterms : 1), sizeof(double complex));
  return S.nn++;
}

static int sp_quadrant(double px, double py, const double c[2]) {
  int q = 0;
  if (px >= c[0]) q += 1;
  if (py <= c[1]) q += 2;
  return q;
}

/* Builds the tree; returns 0, or -1 when a cell at `level_cap` still holds
 * >= num_p blobs (coincident blobs). */
int ora_sp_make_tree(int n, const double *xy, const double *cir, const double *cor, int level_cap) {
  sp_free();
  if (ora_nterms() > 64) return -2; /* the extended evaluation's power table */
  S.nterms = ora_nterms();
  S.num_p = ora_num_p();
  S.theta = ora_theta();
  S.n = n;
  S.x = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  S.y = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  S.cir = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  S.cor = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  for (int i = 0; i < n; i++) {
    S.x[i] = xy[2 * i];
    S.y[i] = xy[2 * i + 1];
    S.cir[i] = cir[i];
    S.cor[i] = cor[i];
  }
  long root = sp_new(0);
  sp_node *r = &S.node[root];
  r->nb = n;
  r->ids = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  for (int i = 0; i < n; i++) r->ids[i] = i;
  if (n > 0) {
    double xmax = S.x[0], xmin = xmax, ymax = S.y[0], ymin = ymax;
    for (int i = 1; i < n; i++) {
      if (S.x[i] > xmax) xmax = S.x[i];
      if (S.x[i] < xmin) xmin = S.x[i];
      if (S.y[i] > ymax) ymax = S.y[i];
      if (S.y[i] < ymin) ymin = S.y[i];
    }
    double rx = fabs(xmax - xmin) + 0.0001;
    double ry = fabs(ymax - ymin) + 0.0001;
    r->region = (rx > ry) ? rx : ry;
    r->c[0] = 0.5 * (xmax + xmin);
    r->c[1] = 0.5 * (ymax + ymin);
  }
  S.levels = 0;
  /* LIFO split from the root (the root is always split) */
  long *stack = NULL, top = -1, scap = 0;
#define PUSH(v)                                                   \
  do {                                                            \
    if (top + 1 == scap) {                                        \
      scap = scap ? 2 * scap : 256;                               \
      stack = (long *)realloc(stack, sizeof(long) * (size_t)scap); \
    }                                                             \
    stack[++top] = (v);                                           \
  } while (0)
  PUSH(root);
  int rc = 0;
  while (top >= 0) {
    long p = stack[top--];
    if (S.node[p].level + 1 > level_cap) {
      rc = -1;
      break;
    }
    long ch[4];
    for (int q = 0; q < 4; q++) ch[q] = sp_new(S.node[p].level + 1);
    sp_node *pn = &S.node[p]; /* after the reallocations */
    for (int q = 0; q < 4; q++) {
      pn->child[q] = ch[q];
      S.node[ch[q]].ids = (int *)malloc(sizeof(int) * (size_t)(pn->nb > 0 ? pn->nb : 1));
    }
    for (int k = 0; k < pn->nb; k++) {
      int id = pn->ids[k];
      sp_node *cn = &S.node[ch[sp_quadrant(S.x[id], S.y[id], pn->c)]];
      cn->ids[cn->nb++] = id;
    }
    for (int q = 0; q < 4; q++) {
      sp_node *cn = &S.node[ch[q]];
      /* the reference sizes each child's list by the parent's count
         (quadtree.c:208-215); only the first nb entries are ever read */
      cn->ids = (int *)realloc(cn->ids, sizeof(int) * (size_t)(cn->nb > 0 ? cn->nb : 1));
      cn->c[0] = (q % 2 != 0) ? pn->c[0] + 0.25 * pn->region : pn->c[0] - 0.25 * pn->region;
      cn->c[1] = (q / 2 == 0) ? pn->c[1] + 0.25 * pn->region : pn->c[1] - 0.25 * pn->region;
      cn->region = 0.5 * pn->region;
      if (cn->level > S.levels) S.levels = cn->level;
      if (cn->nb < S.num_p)
        cn->leaf = 1;
      else
        PUSH(ch[q]);
    }
  }
#undef PUSH
  free(stack);
  if (rc) return rc;
  /* S2M, fmm.c:18-33 */
  for (long i = 0; i < S.nn; i++) {
    sp_node *nd = &S.node[i];
    if (!nd->leaf) continue;
    double complex zc = nd->c[0] + nd->c[1] * I;
    for (int k = 0; k < S.nterms; k++)
      for (int j = 0; j < nd->nb; j++) {
        int b = nd->ids[j];
        double complex zj = S.x[b] + S.y[b] * I;
        nd->a[k] += S.cir[b] * cpow((zj - zc), k);
      }
  }
  /* M2M, fmm.c:35-58: deepest level first, children 3..0, not into the root */
  int nt = S.nterms;
  double complex *acc = (double complex *)malloc(sizeof(double complex) * (size_t)(nt > 0 ? nt : 1));
  for (int lvl = S.levels; lvl >= 2; lvl--) {
    for (long p = 0; p < S.nn; p++) {
      sp_node *pn = &S.node[p];
      if (pn->level != lvl - 1 || pn->child[0] < 0) continue;
      double complex zp = pn->c[0] + pn->c[1] * I;
      for (int q = 3; q >= 0; q--) {
        sp_node *cn = &S.node[pn->child[q]];
        if (cn->nb < 1) continue;
        double complex zc = cn->c[0] + cn->c[1] * I;
        for (int m = 0; m < nt; m++) acc[m] = 0.0;
        for (int m = 0; m < nt; m++)
          for (int k = 0; k < m + 1; k++) {
            long bnm = 1;
            int kk = k > m - k ? m - k : k;
            for (int t = 1; t <= kk; t++) bnm = bnm * (m - kk + t) / t;
            acc[m] += cn->a[k] * (int)bnm * cpow(-(zp - zc), m - k);
          }
        for (int m = 0; m < nt; m++) pn->a[m] += acc[m];
      }
    }
  }
  free(acc);
  return 0;
}

int ora_sp_levels(void) { return S.levels; }
long ora_sp_num_nodes(void) { return S.nn; }

/* ---------------------------------------------------------------------- */
/* FP64 evaluation (the reference's arithmetic)                            */

static void sp_biot_one(double x, double y, double *u, double *v, long *n_m2s, long *n_pairs) {
  double complex phi = 0.0;
  double ud[2] = {0.0, 0.0};
  double complex z = x + y * I;
  long cap = 64, top = 0;
  long *stack = (long *)malloc(sizeof(long) * (size_t)cap);
  stack[0] = 0;
  while (top >= 0) {
    long t = stack[top--];
    const sp_node *nd = &S.node[t];
    if (nd->leaf) {
      double ax = 0.0, ay = 0.0;
      for (int k = 0; k < nd->nb; k++) {
        int b = nd->ids[k];
        double rx = x - S.x[b];
        double ry = y - S.y[b];
        double r = sqrt(pow(rx, 2) + pow(ry, 2));
        if (r > 1.0e-10) {
          double rv2 = 1.0 / pow(r, 2);
          double xai = r / S.cor[b];
          double rv = S.cir[b] * (1.0 - exp(-xai * xai));
          ax -= rv * ry * rv2;
          ay += rv * rx * rv2;
        }
      }
      ud[0] += 0.5 * ax / M_PI;
      ud[1] += 0.5 * ay / M_PI;
      if (n_pairs) *n_pairs += nd->nb;
    } else {
      for (int q = 0; q < 4; q++) {
        long c = nd->child[q];
        const sp_node *cn = &S.node[c];
        double r = sqrt(pow(x - cn->c[0], 2) + pow(y - cn->c[1], 2));
        if (cn->region > S.theta * r) {
          if (top + 1 == cap) {
            cap *= 2;
            stack = (long *)realloc(stack, sizeof(long) * (size_t)cap);
          }
          stack[++top] = c;
        } else {
          double complex zc = cn->c[0] + cn->c[1] * I;
          for (int k = 0; k < S.nterms - 1; k++) phi += cpow((z - zc), (-k - 1)) * cn->a[k];
          if (n_m2s) *n_m2s += 1;
        }
      }
    }
  }
  free(stack);
  phi = 0.5 * (-cimag(phi) + creal(phi) * I) / M_PI;
  *u = -creal(phi) + ud[0];
  *v = cimag(phi) + ud[1];
}

void ora_sp_biot_many(int n, const double *xy, double *uv, int threads, long *n_m2s, long *n_pairs) {
  long m2s_tot = 0, pair_tot = 0;
#ifdef _OPENMP
  if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(threads) reduction(+ : m2s_tot, pair_tot)
#endif
  for (int i = 0; i < n; i++) {
    long a = 0, b = 0;
    if (!S.node) {
      uv[2 * i] = uv[2 * i + 1] = NAN;
      continue;
    }
    sp_biot_one(xy[2 * i], xy[2 * i + 1], &uv[2 * i], &uv[2 * i + 1], &a, &b);
    m2s_tot += a;
    pair_tot += b;
  }
  (void)threads;
  if (n_m2s) *n_m2s = m2s_tot;
  if (n_pairs) *n_pairs = pair_tot;
}

/* ---------------------------------------------------------------------- */
/* extended precision                                                      */

static void sp_make_ext(void) {
  if (S.have_ext) return;
  int nt = S.nterms;
  for (long i = 0; i < S.nn; i++) S.node[i].ae = (ldc *)calloc((size_t)(nt > 0 ? nt : 1), sizeof(ldc));
  for (long i = 0; i < S.nn; i++) {
    sp_node *nd = &S.node[i];
    if (!nd->leaf) continue;
    ldc zc = (long double)nd->c[0] + (long double)nd->c[1] * I;
    for (int j = 0; j < nd->nb; j++) {
      int b = nd->ids[j];
      ldc d = ((long double)S.x[b] + (long double)S.y[b] * I) - zc;
      ldc pk = 1.0L;
      for (int k = 0; k < nt; k++) {
        nd->ae[k] += (long double)S.cir[b] * pk;
        pk *= d;
      }
    }
  }
  for (int lvl = S.levels; lvl >= 2; lvl--) {
    for (long p = 0; p < S.nn; p++) {
      sp_node *pn = &S.node[p];
      if (pn->level != lvl - 1 || pn->child[0] < 0) continue;
      ldc zp = (long double)pn->c[0] + (long double)pn->c[1] * I;
      for (int q = 3; q >= 0; q--) {
        sp_node *cn = &S.node[pn->child[q]];
        if (cn->nb < 1) continue;
        ldc s = ((long double)cn->c[0] + (long double)cn->c[1] * I) - zp;
        ldc sp[64];
        sp[0] = 1.0L;
        for (int j = 1; j < nt; j++) sp[j] = sp[j - 1] * s;
        for (int m = 0; m < nt; m++) {
          ldc acc = 0.0L;
          long double bnm = 1.0L; /* C(m, k), exact in long double */
          for (int k = 0; k <= m; k++) {
            acc += cn->ae[k] * bnm * sp[m - k];
            bnm = bnm * (long double)(m - k) / (long double)(k + 1);
          }
          pn->ae[m] += acc;
        }
      }
    }
  }
  S.have_ext = 1;
}

static void sp_biot_ext_one(double x, double y, double *u, double *v, double *cond) {
  ldc phi = 0.0L;
  long double axs = 0.0L, ays = 0.0L;
  long double mag = 0.0L; /* sum of the contributions' magnitudes */
  const ldc z = (long double)x + (long double)y * I;
  long cap = 64, top = 0;
  long *stack = (long *)malloc(sizeof(long) * (size_t)cap);
  stack[0] = 0;
  while (top >= 0) {
    long t = stack[top--];
    const sp_node *nd = &S.node[t];
    if (nd->leaf) {
      for (int k = 0; k < nd->nb; k++) {
        int b = nd->ids[k];
        /* the pair set is the reference's: r > 1e-10 decided in FP64 */
        double rx = x - S.x[b];
        double ry = y - S.y[b];
        double r = sqrt(pow(rx, 2) + pow(ry, 2));
        if (r > 1.0e-10) {
          long double lx = (long double)x - (long double)S.x[b];
          long double ly = (long double)y - (long double)S.y[b];
          long double r2 = lx * lx + ly * ly;
          long double xai2 = r2 / ((long double)S.cor[b] * (long double)S.cor[b]);
          long double rv = (long double)S.cir[b] * (1.0L - expl(-xai2));
          axs -= rv * ly / r2;
          ays += rv * lx / r2;
          mag += fabsl(rv) / sqrtl(r2);
        }
      }
    } else {
      for (int q = 0; q < 4; q++) {
        long c = nd->child[q];
        const sp_node *cn = &S.node[c];
        double r = sqrt(pow(x - cn->c[0], 2) + pow(y - cn->c[1], 2));
        if (cn->region > S.theta * r) {
          if (top + 1 == cap) {
            cap *= 2;
            stack = (long *)realloc(stack, sizeof(long) * (size_t)cap);
          }
          stack[++top] = c;
        } else {
          ldc w = 1.0L / (z - ((long double)cn->c[0] + (long double)cn->c[1] * I));
          ldc wk = w;
          for (int k = 0; k < S.nterms - 1; k++) {
            phi += wk * cn->ae[k];
            mag += cabsl(wk * cn->ae[k]);
            wk *= w;
          }
        }
      }
    }
  }
  free(stack);
  const long double pi = 3.141592653589793238462643383279502884L;
  *u = (double)((cimagl(phi) + axs) / (2.0L * pi));
  *v = (double)((creall(phi) + ays) / (2.0L * pi));
  if (cond) *cond = (double)(mag / (2.0L * pi));
}

/* The treecode's value at n targets in extended precision (see the file
 * header); uv interleaved, rounded to FP64 at the end.  cond (may be NULL)
 * receives per target the sum of the magnitudes of all its contributions
 * (M2S terms and pairs, over 2 pi): the scale of the rounding error any FP64
 * evaluation of the sum carries, which a cancelling component can be far
 * below. */
void ora_sp_biot_ext(int n, const double *xy, double *uv, double *cond, int threads) {
  if (!S.node) {
    for (int i = 0; i < 2 * n; i++) uv[i] = NAN;
    return;
  }
  sp_make_ext();
#ifdef _OPENMP
  if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
#endif
  for (int i = 0; i < n; i++)
    sp_biot_ext_one(xy[2 * i], xy[2 * i + 1], &uv[2 * i], &uv[2 * i + 1], cond ? &cond[i] : NULL);
  (void)threads;
}

/* ---------------------------------------------------------------------- */
/* dump: the permutation and the non-empty cells below the root in
 * depth-first pre-order, as ora_dump_tree                                 */

typedef struct {
  long pos, cells, cap;
  int *perm, *level, *begin, *end, *leaf;
  double *cx, *cy, *region, *coef;
} sp_dump;

static void sp_dump_rec(long id, sp_dump *d) {
  const sp_node *nd = &S.node[id];
  if (nd->nb < 1) return;
  long slot = -1;
  if (id != 0) {
    slot = d->cells++;
    if (slot < d->cap) {
      d->level[slot] = nd->level;
      d->begin[slot] = (int)d->pos;
      d->leaf[slot] = nd->leaf;
      d->cx[slot] = nd->c[0];
      d->cy[slot] = nd->c[1];
      d->region[slot] = nd->region;
      if (d->coef)
        for (int k = 0; k < S.nterms; k++) {
          d->coef[(slot * S.nterms + k) * 2] = creal(nd->a[k]);
          d->coef[(slot * S.nterms + k) * 2 + 1] = cimag(nd->a[k]);
        }
    }
  }
  if (nd->leaf) {
    for (int k = 0; k < nd->nb; k++) d->perm[d->pos++] = nd->ids[k];
  } else {
    for (int q = 0; q < 4; q++) sp_dump_rec(nd->child[q], d);
  }
  if (slot >= 0 && slot < d->cap) d->end[slot] = (int)d->pos;
}

long ora_sp_dump_tree(int *perm, long cap, int *level, int *begin, int *end, int *leaf, double *cx, double *cy,
                      double *region, double *coef) {
  if (!S.node) return -1;
  int *tmp = NULL;
  if (!perm) tmp = perm = (int *)malloc(sizeof(int) * (size_t)(S.n > 0 ? S.n : 1));
  sp_dump d = {0, 0, cap, perm, level, begin, end, leaf, cx, cy, region, coef};
  sp_dump_rec(0, &d);
  free(tmp);
  return d.cells;
}

void ora_sp_reset(void) { sp_free(); }
