/*
 * ref_driver.c -- runs the reference treecode, built from its own sources
 * (ver-c/src/{quadtree,fmm,morton_order}.c, left where they lie), on one
 * input file and writes what it computed.  TEST INFRASTRUCTURE ONLY: it
 * generates the golden vectors that pin the oracle, and is never part of
 * the product.
 *
 * Usage:  ref_driver <input.bin> <output.bin> [threads] [batches]
 * With batches > 1 the targets are evaluated that many times over the same
 * tree (a timed CPU baseline); every batch's time is printed.
 * The reference reads its parameters from ../cal_cond/fmm_param.dat
 * relative to the working directory (quadtree.c:12-27), so the caller runs
 * this program from a directory that has that file beside it.
 *
 * input.bin : int32 n, int32 ntgt, f64 xy[n][2], f64 cir[n], f64 cor[n],
 *             f64 txy[ntgt][2]
 * output.bin: int32 n, ntgt, ncells, nterms, max_level,
 *             f64 uv[ntgt][2], int32 perm[n],
 *             int32 level/begin/end/leaf[ncells], f64 cx/cy/region[ncells],
 *             f64 coef[ncells][nterms][2]
 * Cells are the non-empty cells below the root in depth-first pre-order,
 * quadrants 0..3; the permutation lists the blobs of the leaves in that order.
 */
#include <complex.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "fmm.h"
#include "morton_order.h"
#include "quadtree.h"

static int *g_perm, g_pos;
static long g_nc, g_cap;
static int *g_level, *g_begin, *g_end, *g_leaf;
static double *g_cx, *g_cy, *g_region, *g_coef;

static void walk(int id) {
  Node *nd = &qtree.node[id];
  if (nd->num_vor < 1) return;
  long slot = -1;
  if (id != 0) {
    slot = g_nc++;
    if (slot < g_cap) {
      g_level[slot] = nd->level;
      g_begin[slot] = g_pos;
      g_leaf[slot] = nd->is_leaf;
      g_cx[slot] = nd->center_pos[0];
      g_cy[slot] = nd->center_pos[1];
      g_region[slot] = nd->region;
      for (int k = 0; k < qtree.nterms; k++) {
        g_coef[(slot * qtree.nterms + k) * 2] = creal(nd->outer_coeffs[k]);
        g_coef[(slot * qtree.nterms + k) * 2 + 1] = cimag(nd->outer_coeffs[k]);
      }
    }
  }
  if (nd->is_leaf) {
    for (int k = 0; k < nd->num_vor; k++) g_perm[g_pos++] = nd->vor_id[k];
  } else {
    int ch[4];
    getChild(id, ch);
    for (int q = 0; q < 4; q++) walk(ch[q]);
  }
  if (slot >= 0 && slot < g_cap) g_end[slot] = g_pos;
}

static double now(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

int main(int argc, char **argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: %s in.bin out.bin [threads]\n", argv[0]);
    return 2;
  }
  int threads = argc > 3 ? atoi(argv[3]) : 1;
  int batches = argc > 4 ? atoi(argv[4]) : 1;
  if (batches < 1) batches = 1;
  FILE *f = fopen(argv[1], "rb");
  if (!f) return 3;
  int n, nt;
  if (fread(&n, 4, 1, f) != 1 || fread(&nt, 4, 1, f) != 1) return 4;
  double *xy = malloc(sizeof(double) * 2 * (size_t)n);
  double *cir = malloc(sizeof(double) * (size_t)n);
  double *cor = malloc(sizeof(double) * (size_t)n);
  double *txy = malloc(sizeof(double) * 2 * (size_t)(nt > 0 ? nt : 1));
  double *uv = malloc(sizeof(double) * 2 * (size_t)(nt > 0 ? nt : 1));
  if (fread(xy, 8, 2 * (size_t)n, f) != 2 * (size_t)n) return 5;
  if (fread(cir, 8, (size_t)n, f) != (size_t)n) return 5;
  if (fread(cor, 8, (size_t)n, f) != (size_t)n) return 5;
  if (fread(txy, 8, 2 * (size_t)nt, f) != 2 * (size_t)nt) return 5;
  fclose(f);

  double t0 = now();
  make_tree(n, (void *)xy, cir, cor);
  double t1 = now(), t2 = t1;
  for (int rep = 0; rep < batches; rep++) {
    double tb = now();
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
#endif
    for (int i = 0; i < nt; i++) biot_tree(txy[2 * i], txy[2 * i + 1], &uv[2 * i], &uv[2 * i + 1]);
    t2 = now();
    if (batches > 1) fprintf(stderr, "ref: batch %d biot_tree %.6f s\n", rep, t2 - tb);
  }
  fprintf(stderr, "ref: n=%d ntgt=%d make_tree %.4f s, biot_tree %.4f s (%d threads), max_level %d\n",
          n, nt, t1 - t0, (t2 - t1) / batches, threads, qtree.max_level);

  /* count, then dump */
  g_perm = malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  g_cap = 0;
  g_pos = 0;
  g_nc = 0;
  walk(0);
  long nc = g_nc;
  g_cap = nc;
  g_level = malloc(4 * (size_t)(nc + 1));
  g_begin = malloc(4 * (size_t)(nc + 1));
  g_end = malloc(4 * (size_t)(nc + 1));
  g_leaf = malloc(4 * (size_t)(nc + 1));
  g_cx = malloc(8 * (size_t)(nc + 1));
  g_cy = malloc(8 * (size_t)(nc + 1));
  g_region = malloc(8 * (size_t)(nc + 1));
  g_coef = malloc(16 * (size_t)(nc + 1) * (size_t)qtree.nterms);
  g_pos = 0;
  g_nc = 0;
  walk(0);

  FILE *o = fopen(argv[2], "wb");
  if (!o) return 6;
  int hdr[5] = {n, nt, (int)nc, qtree.nterms, qtree.max_level};
  fwrite(hdr, 4, 5, o);
  fwrite(uv, 8, 2 * (size_t)nt, o);
  fwrite(g_perm, 4, (size_t)n, o);
  fwrite(g_level, 4, (size_t)nc, o);
  fwrite(g_begin, 4, (size_t)nc, o);
  fwrite(g_end, 4, (size_t)nc, o);
  fwrite(g_leaf, 4, (size_t)nc, o);
  fwrite(g_cx, 8, (size_t)nc, o);
  fwrite(g_cy, 8, (size_t)nc, o);
  fwrite(g_region, 8, (size_t)nc, o);
  fwrite(g_coef, 16, (size_t)nc * (size_t)qtree.nterms, o);
  fclose(o);
  return 0;
}
