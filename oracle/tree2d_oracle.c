/*
 * tree2d_oracle.c -- CPU oracle for the 2-D vortex-blob treecode.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this file.  It is used by the test-suite as the checker, by
 * `__graft_entry__.smoke()` as the checker, and by `bench.py` as the timed
 * CPU baseline ("port" of the reference CPU implementation).
 *
 * It restates, in plain C, the algorithm of the reference implementation
 * (yukihirabayasi/2DFMM, ver-c/src):
 *
 *   - root box ............ ver-c/src/quadtree.c:81-99   (calc_region)
 *   - quadrant test ....... ver-c/src/quadtree.c:29-35   (quadrant_pos)
 *   - child centres ....... ver-c/src/quadtree.c:61-79   (calc_CenterPos)
 *   - max-level search .... ver-c/src/quadtree.c:102-171 (make_tree)
 *   - LIFO cell splitting . ver-c/src/quadtree.c:173-251 (split_cell)
 *   - level-order ids ..... ver-c/src/morton_order.c:4-51
 *   - S2M ................. ver-c/src/fmm.c:18-33
 *   - M2M ................. ver-c/src/fmm.c:35-58
 *   - M2S ................. ver-c/src/fmm.c:60-67
 *   - per-target traversal  ver-c/src/fmm.c:69-118       (biot_tree)
 *   - regularised P2P ..... ver-c/src/fmm.c:121-142      (direct_evaluate)
 *
 * The data layout is the reference's: a dense, complete quadtree of
 * (4^(L+1)-1)/3 nodes in level order, a max-level that persists between
 * calls and grows by one per failed attempt, and a per-call traversal stack
 * of num_nodes int entries (the split and the traversal stacks are -1-filled
 * ints, quadtree.c:183-188 and fmm.c:83-87).  Those choices are kept on
 * purpose: they set the reference's cost, and this file doubles as its
 * timed CPU stand-in where the reference's own build is not available.
 *
 * Every floating-point expression that decides a result is written in the
 * same form as the reference (complex arithmetic, cpow for powers, pow(.,2)
 * in the distances, the same summation order), because the oracle is held
 * bit-exact against the reference built from its own sources.  Compile with
 * -ffp-contract=off so that no platform fuses those expressions.
 *
 * Also here: the FP64 direct O(N*M) sum that measures approximate results; it
 * applies the regularised kernel of direct_evaluate (fmm.c:121-142, r > 1e-10)
 * to every source, i.e. biot_b of ver-c/src/includes/d_biot.f90:2-64 with the
 * path's threshold.
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

typedef struct {
  double pos[2];
  double cir;
  double cor;
} ora_blob;

typedef struct {
  int level;
  int nb;            /* number of blobs in the cell                 */
  int *ids;          /* blob ids, in the order they were bucketed    */
  double c[2];       /* centre                                       */
  double region;     /* side length                                  */
  double complex *a; /* outer (Laurent) coefficients, nterms         */
  int leaf;
  int made;          /* 1 once the cell was created by a split       */
} ora_node;

static struct {
  int nterms, num_p;
  double theta, r_min;
  int have_params;
  int max_level;     /* persists between calls, like quadtree.c:109  */
  int levels;        /* max level of the current tree                */
  long num_nodes;
  ora_node *node;
  ora_blob *blob;
  int nblob;
} g;

/* ---------------------------------------------------------------------- */
/* level-order index algebra of a complete quadtree (morton_order.c:4-51)  */

static long level_offset(int level) { return ((1L << (2 * level)) - 1) / 3; }

static void children_of(long id, int level, long out[4]) {
  long local = id - level_offset(level);
  for (int q = 0; q < 4; q++) out[q] = level_offset(level + 1) + 4 * local + q;
}

static long parent_of(long id, int level) {
  return level_offset(level - 1) + ((id - level_offset(level)) >> 2);
}

/* Exported for known-answer tests of the index algebra. */
int ora_level_of(long id) {
  int l = 0;
  while (level_offset(l + 1) <= id) l++;
  return l;
}
long ora_child(long id, int q) {
  long ch[4];
  children_of(id, ora_level_of(id), ch);
  return ch[q & 3];
}
long ora_parent(long id) { return parent_of(id, ora_level_of(id)); }
long ora_global2local(long id, int level) { return id - level_offset(level); }

/* ---------------------------------------------------------------------- */
/* parameters                                                              */

int ora_set_params(int nterms, int num_p, double theta, double r_min) {
  g.nterms = nterms;
  g.num_p = num_p;
  g.theta = theta;
  g.r_min = r_min;
  g.have_params = 1;
  return 0;
}

/* Resets the persistent max-level search state (a fresh process in the
 * reference starts at 1). */
void ora_reset(void) { g.max_level = 1; }

static void free_tree(void);
/* Releases the tree (the dense array can take tens of GB). */
void ora_free(void) { free_tree(); }

/* ---------------------------------------------------------------------- */
/* tree construction                                                       */

static void free_tree(void) {
  if (g.node) {
    for (long i = 0; i < g.num_nodes; i++) {
      free(g.node[i].ids);
      free(g.node[i].a);
    }
    free(g.node);
  }
  g.node = NULL;
  g.num_nodes = 0;
}

static int quadrant(const double p[2], const double c[2]) {
  int q = 0;
  if (p[0] >= c[0]) q += 1;
  if (p[1] <= c[1]) q += 2;
  return q;
}

int ora_quadrant(double px, double py, double cx, double cy) {
  double p[2] = {px, py}, c[2] = {cx, cy};
  return quadrant(p, c);
}

static void child_centre(int q, const double pc[2], double region, double cc[2]) {
  cc[0] = (q % 2 != 0) ? pc[0] + 0.25 * region : pc[0] - 0.25 * region;
  cc[1] = (q / 2 == 0) ? pc[1] + 0.25 * region : pc[1] - 0.25 * region;
}

static void root_box(ora_node *root) {
  int n = g.nblob;
  double xmax = g.blob[0].pos[0], xmin = xmax, ymax = g.blob[0].pos[1], ymin = ymax;
  for (int i = 1; i < n; i++) {
    double x = g.blob[i].pos[0], y = g.blob[i].pos[1];
    if (x > xmax) xmax = x;
    if (x < xmin) xmin = x;
    if (y > ymax) ymax = y;
    if (y < ymin) ymin = y;
  }
  double rx = fabs(xmax - xmin) + 0.0001;
  double ry = fabs(ymax - ymin) + 0.0001;
  root->region = (rx > ry) ? rx : ry;
  root->c[0] = 0.5 * (xmax + xmin);
  root->c[1] = 0.5 * (ymax + ymin);
}

/* One attempt at max level L.  Returns 0 on success, -1 if a cell that must
 * be split sits at level L. */
static int build_attempt(int L) {
  free_tree();
  g.levels = L;
  g.num_nodes = level_offset(L + 1);
  g.node = (ora_node *)calloc((size_t)g.num_nodes, sizeof(ora_node));
  if (!g.node) return -2;
  for (int l = 0; l <= L; l++)
    for (long i = level_offset(l); i < level_offset(l + 1); i++) g.node[i].level = l;

  ora_node *root = &g.node[0];
  root->nb = g.nblob;
  root->made = 1;
  root->a = (double complex *)calloc((size_t)g.nterms, sizeof(double complex));
  root->ids = (int *)malloc(sizeof(int) * (size_t)(g.nblob > 0 ? g.nblob : 1));
  for (int i = 0; i < g.nblob; i++) root->ids[i] = i;
  if (g.nblob > 0) root_box(root);

  /* an int stack of num_nodes entries, -1-filled, as quadtree.c:183-188 */
  int *stack = (int *)malloc(sizeof(int) * (size_t)g.num_nodes);
  stack[0] = 0;
  for (long i = 1; i < g.num_nodes; i++) stack[i] = -1;
  long top = 0;
  int rc = 0;
  while (top >= 0) {
    long p = stack[top];
    stack[top--] = -1;
    ora_node *pn = &g.node[p];
    if (pn->level + 1 > L) {
      rc = -1;
      break;
    }
    long ch[4];
    children_of(p, pn->level, ch);
    for (int q = 0; q < 4; q++) {
      ora_node *cn = &g.node[ch[q]];
      cn->ids = (int *)malloc(sizeof(int) * (size_t)(pn->nb > 0 ? pn->nb : 1));
      cn->nb = 0;
    }
    for (int k = 0; k < pn->nb; k++) {
      int id = pn->ids[k];
      ora_node *cn = &g.node[ch[quadrant(g.blob[id].pos, pn->c)]];
      cn->ids[cn->nb++] = id;
    }
    for (int q = 0; q < 4; q++) {
      ora_node *cn = &g.node[ch[q]];
      child_centre(q, pn->c, pn->region, cn->c);
      cn->level = pn->level + 1;
      cn->region = 0.5 * pn->region;
      cn->made = 1;
      cn->a = (double complex *)calloc((size_t)g.nterms, sizeof(double complex));
      if (cn->nb < g.num_p)
        cn->leaf = 1;
      else
        stack[++top] = (int)ch[q];
    }
  }
  free(stack);
  return rc;
}

/* S2M, fmm.c:18-33: a_k = sum_j cir_j (z_j - z_c)^k over a leaf's blobs. */
static void s2m(void) {
  for (long i = 0; i < g.num_nodes; i++) {
    ora_node *nd = &g.node[i];
    if (!nd->leaf) continue;
    double complex zc = nd->c[0] + nd->c[1] * I;
    for (int k = 0; k < g.nterms; k++) {
      for (int j = 0; j < nd->nb; j++) {
        const ora_blob *b = &g.blob[nd->ids[j]];
        double complex zj = b->pos[0] + b->pos[1] * I;
        nd->a[k] += b->cir * cpow((zj - zc), k);
      }
    }
  }
}

static int binom(int n, int k) {
  /* exact binomial coefficient (the reference's recursive `combination`) */
  long r = 1;
  if (k < 0 || k > n) return 0;
  if (k > n - k) k = n - k;
  for (int i = 1; i <= k; i++) r = r * (n - k + i) / i;
  return (int)r;
}

/* M2M, fmm.c:35-58: sibling groups in descending id order (deepest level
 * first, quadrant 3 down to 0); the level-1 -> root shift is not done. */
static void m2m(void) {
  int nt = g.nterms;
  double complex *acc = (double complex *)malloc(sizeof(double complex) * (size_t)nt);
  for (long last = g.num_nodes - 1; last > 4; last -= 4) {
    int lvl = g.node[last].level;
    long p = parent_of(last, lvl);
    double complex zp = g.node[p].c[0] + g.node[p].c[1] * I;
    for (long c = last; c > last - 4; c--) {
      ora_node *cn = &g.node[c];
      if (cn->nb < 1) continue;
      double complex zc = cn->c[0] + cn->c[1] * I;
      for (int n = 0; n < nt; n++) acc[n] = 0.0;
      for (int n = 0; n < nt; n++)
        for (int k = 0; k < n + 1; k++)
          acc[n] += cn->a[k] * binom(n, k) * cpow(-(zp - zc), n - k);
      for (int n = 0; n < nt; n++) g.node[p].a[n] += acc[n];
    }
  }
  free(acc);
}

/* Parameter file, read the way quadtree.c:12-27 reads it: four fscanf
 * conversions, each result ignored (a Fortran-style "0.5d0" stops the
 * scan after "0.5", so r_min is then left as it was; r_min is unused). */
static int read_param_file(const char *path) {
  FILE *f = fopen(path, "r");
  if (!f) return -1;
  if (fscanf(f, "%i    nterms", &g.nterms) < 0) { /* ignored */ }
  if (fscanf(f, "%i   num_p", &g.num_p) < 0) { /* ignored */ }
  if (fscanf(f, "%lf theta", &g.theta) < 0) { /* ignored */ }
  if (fscanf(f, "%lf  r_min ! for Tree", &g.r_min) < 0) { /* ignored */ }
  fclose(f);
  g.have_params = 1;
  return 0;
}

/* make_tree (quadtree.c:102-171).  xy holds x,y interleaved per blob.
 * Parameters come from ora_set_params, or from `param_file` when non-NULL.
 * Returns 0, or <0 when the tree cannot be built (max_level_cap exceeded). */
int ora_make_tree(int n, const double *xy, const double *cir, const double *cor,
                  const char *param_file, int max_level_cap) {
  if (param_file && read_param_file(param_file) != 0) return -3;
  if (!g.have_params) return -4;
  if (g.max_level < 1) g.max_level = 1;
  free(g.blob);
  g.nblob = n;
  g.blob = (ora_blob *)malloc(sizeof(ora_blob) * (size_t)(n > 0 ? n : 1));
  for (int i = 0; i < n; i++) {
    g.blob[i].pos[0] = xy[2 * i];
    g.blob[i].pos[1] = xy[2 * i + 1];
    g.blob[i].cir = cir[i];
    g.blob[i].cor = cor[i];
  }
  for (;;) {
    if (g.max_level > max_level_cap) return -1;
    int rc = build_attempt(g.max_level);
    if (rc == 0) break;
    if (rc == -2) return -2;
    g.max_level++;
  }
  s2m();
  m2m();
  return 0;
}

/* ---------------------------------------------------------------------- */
/* evaluation                                                              */

/* M2S, fmm.c:60-67 */
static void m2s(double complex z, double complex *phi, const ora_node *nd) {
  double complex zc = nd->c[0] + nd->c[1] * I;
  for (int k = 0; k < g.nterms - 1; k++) *phi += cpow((z - zc), (-k - 1)) * nd->a[k];
}

/* direct_evaluate, fmm.c:121-142 */
static void p2p(double x, double y, const ora_node *nd, double ud[2]) {
  double ax = 0.0, ay = 0.0;
  for (int k = 0; k < nd->nb; k++) {
    const ora_blob *b = &g.blob[nd->ids[k]];
    double rx = x - b->pos[0];
    double ry = y - b->pos[1];
    double r = sqrt(pow(rx, 2) + pow(ry, 2));
    if (r > 1.0e-10) {
      double rv2 = 1.0 / pow(r, 2);
      double xai = r / b->cor;
      double rv = b->cir * (1.0 - exp(-xai * xai));
      ax -= rv * ry * rv2;
      ay += rv * rx * rv2;
    }
  }
  ud[0] += 0.5 * ax / M_PI;
  ud[1] += 0.5 * ay / M_PI;
}

/* biot_tree, fmm.c:69-118: LIFO traversal from the root; per child the
 * acceptance test region > theta*r decides descend (push) or M2S.  The
 * stack has num_nodes entries and is allocated per call, as in the
 * reference.  Work counters are optional (NULL to skip). */
static void biot_one(double x, double y, double *u, double *v, long *n_m2s, long *n_pairs) {
  double complex phi = 0.0;
  double ud[2] = {0.0, 0.0};
  /* an int stack of num_nodes entries, -1-filled, per call (fmm.c:83-87) */
  int *stack = (int *)malloc(sizeof(int) * (size_t)g.num_nodes);
  stack[0] = 0;
  for (long i = 1; i < g.num_nodes; i++) stack[i] = -1;
  long top = 0;
  double complex z = x + y * I;
  while (top >= 0) {
    long t = stack[top];
    stack[top--] = -1;
    const ora_node *nd = &g.node[t];
    if (nd->leaf) {
      p2p(x, y, nd, ud);
      if (n_pairs) *n_pairs += nd->nb;
    } else {
      long ch[4];
      children_of(t, nd->level, ch);
      for (int q = 0; q < 4; q++) {
        const ora_node *cn = &g.node[ch[q]];
        double r = sqrt(pow(x - cn->c[0], 2) + pow(y - cn->c[1], 2));
        if (cn->region > g.theta * r) {
          stack[++top] = (int)ch[q];
        } else {
          m2s(z, &phi, cn);
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

void ora_biot_tree(double x, double y, double *u, double *v) {
  if (!g.node) {
    *u = NAN;
    *v = NAN;
    return;
  }
  biot_one(x, y, u, v, NULL, NULL);
}

/* Evaluates n targets (xy interleaved) into uv (interleaved), with up to
 * `threads` OpenMP threads (<=0: all).  Counters (may be NULL) receive the
 * total accepted-cell and direct-pair counts. */
void ora_biot_many(int n, const double *xy, double *uv, int threads, long *n_m2s, long *n_pairs) {
  long m2s_tot = 0, pair_tot = 0;
#ifdef _OPENMP
  if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(threads) reduction(+ : m2s_tot, pair_tot)
#endif
  for (int i = 0; i < n; i++) {
    long a = 0, b = 0;
    if (!g.node) {
      uv[2 * i] = NAN;
      uv[2 * i + 1] = NAN;
      continue;
    }
    biot_one(xy[2 * i], xy[2 * i + 1], &uv[2 * i], &uv[2 * i + 1], &a, &b);
    m2s_tot += a;
    pair_tot += b;
  }
  (void)threads;
  if (n_m2s) *n_m2s = m2s_tot;
  if (n_pairs) *n_pairs = pair_tot;
}

/* ---------------------------------------------------------------------- */
/* introspection for parity tests                                          */

int ora_levels(void) { return g.levels; }
long ora_num_nodes(void) { return g.num_nodes; }
int ora_nterms(void) { return g.nterms; }
int ora_num_p(void) { return g.num_p; }
double ora_theta(void) { return g.theta; }

typedef struct {
  long *perm_pos; /* running write position into perm */
  int *perm;
  long cells, cap;
  int *level, *begin, *end, *leaf;
  double *cx, *cy, *region;
  double *coef; /* cells x nterms x 2 */
} ora_dump;

static void dump_rec(long id, ora_dump *d) {
  const ora_node *nd = &g.node[id];
  if (nd->nb < 1) return; /* empty cells carry no blobs and zero coefficients */
  long slot = -1;
  if (id != 0) {
    slot = d->cells++;
    if (slot < d->cap) {
      d->level[slot] = nd->level;
      d->begin[slot] = (int)*d->perm_pos;
      d->leaf[slot] = nd->leaf;
      d->cx[slot] = nd->c[0];
      d->cy[slot] = nd->c[1];
      d->region[slot] = nd->region;
      if (d->coef)
        for (int k = 0; k < g.nterms; k++) {
          d->coef[(slot * g.nterms + k) * 2] = creal(nd->a[k]);
          d->coef[(slot * g.nterms + k) * 2 + 1] = cimag(nd->a[k]);
        }
    }
  }
  if (nd->leaf) {
    for (int k = 0; k < nd->nb; k++) d->perm[(*d->perm_pos)++] = nd->ids[k];
  } else {
    long ch[4];
    children_of(id, nd->level, ch);
    for (int q = 0; q < 4; q++) dump_rec(ch[q], d);
  }
  if (slot >= 0 && slot < d->cap) d->end[slot] = (int)*d->perm_pos;
}

/* Writes the blob permutation (leaves in depth-first quadrant order 0..3,
 * blobs in bucketing order inside a leaf) and the non-empty cells below the
 * root in depth-first pre-order.  Returns the number of cells (the arrays
 * must hold `cap` entries; call with cap=0 to count). */
long ora_dump_tree(int *perm, long cap, int *level, int *begin, int *end, int *leaf, double *cx,
                   double *cy, double *region, double *coef) {
  if (!g.node) return -1;
  long pos = 0;
  int *tmp = NULL;
  if (!perm) tmp = perm = (int *)malloc(sizeof(int) * (size_t)(g.nblob > 0 ? g.nblob : 1));
  ora_dump d = {&pos, perm, 0, cap, level, begin, end, leaf, cx, cy, region, coef};
  dump_rec(0, &d);
  free(tmp);
  return d.cells;
}

/* ---------------------------------------------------------------------- */
/* FP64 direct sum (the accuracy yardstick)                                             */

void ora_direct(int ntgt, const double *txy, int nsrc, const double *sxy, const double *cir,
                const double *cor, double *uv, int threads) {
#ifdef _OPENMP
  if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
#endif
  for (int i = 0; i < ntgt; i++) {
    double x = txy[2 * i], y = txy[2 * i + 1];
    double ax = 0.0, ay = 0.0;
    for (int j = 0; j < nsrc; j++) {
      double rx = x - sxy[2 * j];
      double ry = y - sxy[2 * j + 1];
      double r = sqrt(rx * rx + ry * ry);
      if (r > 1.0e-10) {
        double rv2 = 1.0 / (r * r);
        double xai = r / cor[j];
        double rv = cir[j] * (1.0 - exp(-xai * xai));
        ax -= rv * ry * rv2;
        ay += rv * rx * rv2;
      }
    }
    uv[2 * i] = 0.5 * ax / M_PI;
    uv[2 * i + 1] = 0.5 * ay / M_PI;
  }
  (void)threads;
}

int ora_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
