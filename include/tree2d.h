/*
 * tree2d.h -- C ABI of the GB300 vortex-blob treecode (libtree2d_gb300.so).
 *
 * Drop-in replacement for the reference's two entry points and the Fortran
 * bind(C) interface that calls them:
 *
 *   make_tree  <- ver-c/src/quadtree.c:102-171 (declared quadtree.h:38-41)
 *   biot_tree  <- ver-c/src/fmm.c:69-118       (declared fmm.h:7)
 *   Fortran    <- ver-c/src/m_tree_bindc.f90:1-17 (module m_tree_bindc)
 *
 * All other symbols are additive extensions; a caller written for the
 * reference needs none of them.  All functions use plain C types; there are
 * no CUDA or library types in any signature (streams are passed as void*).
 *
 * Threading: make_tree and the tree2d_* calls that change state must not
 * run concurrently with any other call.  biot_tree and biot_tree_batch may
 * be called from several threads at once after make_tree returned.
 */
#ifndef TREE2D_GB300_H
#define TREE2D_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ */
/* Reference entry points                                              */

/* Builds the tree over nvor_b vortex blobs and evaluates the velocity at
 * every blob position.  vor_b holds x,y interleaved per blob (C
 * double[nvor_b][2] == Fortran vor_b(2,nvor_b)); cir_b the circulations,
 * cor_b the core radii.  Inputs are copied; the caller may reuse them at
 * once.  Parameters come from ../cal_cond/fmm_param.dat relative to the
 * working directory, as in the reference (quadtree.c:12-27), unless
 * tree2d_set_params() fixed them.  Replaces quadtree.c:102 make_tree.
 * Errors: none returned (the reference returns void); see
 * tree2d_last_error().  After a failed call biot_tree returns NaN. */
void make_tree(int nvor_b, const double *vor_b, const double *cir_b, const double *cor_b);

/* Velocity (u,v) induced at (x,y) by the blobs of the last make_tree.
 * Replaces fmm.c:69 biot_tree.  Positions equal (bit for bit) to a blob
 * position are answered from the velocities make_tree computed; any other
 * point is evaluated on the GPU by the same traversal.  Without a valid
 * tree, u and v are set to NaN. */
void biot_tree(double x, double y, double *u, double *v);

/* ------------------------------------------------------------------ */
/* Extensions                                                          */

/* Status codes (tree2d_last_error). */
#define TREE2D_OK 0
#define TREE2D_ERR_PARAM_FILE 1    /* parameter file missing and no override      */
#define TREE2D_ERR_BAD_PARAMS 2    /* an argument outside its call's range; for
                                      tree2d_set_params: nterms outside 0..32, num_p
                                      outside 2..65536, or a non-finite theta       */
#define TREE2D_ERR_BAD_INPUT 3     /* n < 0, or non-finite position/cir/cor        */
#define TREE2D_ERR_TOO_DEEP 4      /* >= num_p blobs share one cell at level 32    */
#define TREE2D_ERR_CUDA 5          /* CUDA runtime or kernel failure               */
#define TREE2D_ERR_NO_TREE 6       /* evaluation requested before a valid tree     */
#define TREE2D_ERR_NO_DEVICE 7     /* no CUDA device                               */
#define TREE2D_ERR_TIMEOUT 8       /* a bounded device loop gave up                */
#define TREE2D_ERR_MODE 9          /* unknown mode, or a call that the mode or the
                                      settings in force do not support              */
#define TREE2D_ERR_TOO_LARGE 10    /* beyond the fixed scratch of the static solve,
                                      or more than 2^31 - 1 interaction-list entries */
#define TREE2D_ERR_FILE 11         /* a file could not be read or has the wrong format */

/* Evaluation modes (tree2d_set_mode). */
#define TREE2D_MODE_PLAIN 0        /* FP64 treecode, reference semantics             */
#define TREE2D_MODE_MIXED 1        /* scaled FP32 FMM, tensor-core M2L, FP64 final sum */
#define TREE2D_MODE_LEARNED 2      /* MIXED with learned per-interaction order         */

int tree2d_last_error(void);
const char *tree2d_error_string(int code);

/* Fixes the parameters (nterms = stored coefficients, num_p = leaf split
 * threshold, theta = opening angle, r_min unused as in the reference) so
 * that make_tree no longer reads the parameter file.  Returns a status. */
int tree2d_set_params(int nterms, int num_p, double theta, double r_min);
/* Returns make_tree to reading ../cal_cond/fmm_param.dat. */
void tree2d_clear_params(void);
/* Reads the parameters in force (after the last make_tree). */
void tree2d_get_params(int *nterms, int *num_p, double *theta, double *r_min);

int tree2d_set_mode(int mode);
int tree2d_get_mode(void);

/* Parameters of the mixed form: expansion length pterms (2..32) of its
 * multipole and local expansions, the radius of the regularisation
 * correction in units of the largest core radius (pairs closer than that
 * which the far field treats as point vortices get exp(-r^2/sigma^2)
 * added back), and whether M2L runs on the tensor cores (1) or on CUDA
 * cores (0, for checking).  Defaults 16, 2.5, 1. */
int tree2d_set_mixed_params(int pterms, double cutoff_sigmas, int use_tensor_cores);

/* Most blobs per leaf of the tree the mixed and learned forms build (the
 * plain form always uses the parameters' num_p - 1, as the reference does):
 * -1 (the default) chooses by the blobs per set: 96 below 2,097,152, 128
 * above (a batched solve uses its mean set size); 0 uses num_p - 1;
 * 1..65535 fixes it. */
int tree2d_set_mixed_leaf(int max_blobs);

/* Evaluates n targets (xy interleaved, host memory) into uv (interleaved,
 * host memory) against the last make_tree.  Blob positions are answered
 * from the precomputed velocities, the rest in one GPU launch.  The points
 * are matched on the GPU (target i against blob i, bit for bit; page-locked
 * xy and uv let the copies overlap), the others through a host table.
 * Returns a status; on error uv is filled with NaN. */
int biot_tree_batch(int n, const double *xy, double *uv);

/* Device-resident solve: builds the tree over n blobs whose arrays are in
 * device memory (xy interleaved f64, cir f64, cor f64) and writes the
 * velocity at every blob position into d_uv (interleaved, original blob
 * order), all on `stream` (a cudaStream_t, or NULL for the legacy default
 * stream).  Uses the parameters and mode in force.  It does not change the
 * state seen by biot_tree.  Returns a status. */
int tree2d_solve_device(int n, const double *d_xy, const double *d_cir, const double *d_cor,
                        double *d_uv, void *stream);

/* The plain-mode solve of tree2d_solve_device (same kernels, same results
 * bit for bit), for callers that cannot allocate GPU memory: a host program
 * whose device memory belongs to a pool it must not go around, or an
 * embedding that fixes its memory footprint at start-up.  The call
 * allocates nothing: all scratch lives in one 32 MiB file-scope device
 * array per GPU, resident until the process exits.  The caller still passes
 * inputs and outputs.  Plain form only: with TREE2D_MODE_MIXED or
 * TREE2D_MODE_LEARNED in force, or a mirror wall set (tree2d_set_mirror),
 * it returns TREE2D_ERR_MODE and computes nothing.  Limits: n <= 65536
 * blobs and as many cells as fit in the array; beyond that it returns
 * TREE2D_ERR_TOO_LARGE.  Every call shares the array and it keeps the last
 * call's contents (what the solve reads it clears first); calls that
 * overlap on the GPU race, so do not run two at once on different streams.
 * The first call on a device looks up the array's device address; make it
 * before any stream capture.  It returns after its work on `stream` is done.
 * No counterpart in the reference. */
int tree2d_solve_device_static(int n, const double *d_xy, const double *d_cir, const double *d_cor,
                               double *d_uv, void *stream);

/* Statistics of the last solve (make_tree or tree2d_solve_device). */
typedef struct {
  long long n_blobs;
  long long n_cells;      /* non-empty cells, root included          */
  long long n_leaves;
  int depth;              /* deepest leaf level                      */
  int mode;
  long long n_m2s;        /* accepted (target, cell) pairs            */
  long long n_pairs;      /* direct (target, source) pairs            */
  long long n_m2l;        /* M2L (target cell, source cell) pairs     */
  double ms_build;        /* device time of the tree build            */
  double ms_upward;       /* plain: S2M + M2M; mixed: lists, upward
                             pass, M2L, P2L, L2L                      */
  double ms_eval;         /* evaluation at the targets (one kernel)   */
  double ms_total;
  long long n_launches;   /* kernels launched by the solve            */
  int m2l_path;           /* mixed: 1 = CUDA cores, 2 = tensor cores  */
  int eval_variant;       /* mixed: near-field kernel variant that ran
                             (0/1: global loads, 4/8 warps per block;
                              2/3: blobs staged by bulk copies, 4/8)    */
  int learned_active;     /* learned: 1 if the network's decisions were
                             applied, 0 if the solve ran the fixed mixed
                             form (no weights, or lists outside the
                             network's training envelope)               */
  long long n_list_u;     /* mixed: U (direct) list entries             */
  long long n_list_k;     /* mixed: K (correction) list entries         */
  int leaf_blobs;         /* most blobs per leaf of the tree built        */
  long long n_list_k_blobs; /* mixed: source blobs of the K lists, summed
                             over the leaves; learned: out to the
                             envelope's radius (the envelope statistic) */
  long long n_pairs_k;    /* mixed: correction pairs evaluated (part of
                             n_pairs; the rest are direct U pairs)      */
  long long n_pairs_k_listed; /* mixed: pairs of the correction entries
                             evaluated, before 16-blob chunks farther than
                             the correction radius were skipped          */
  int m2l_rows;           /* mixed, tensor-core M2L: cells per CTA of the
                             solve (128 or 64)                          */
} tree2d_stats_t;
int tree2d_get_stats(tree2d_stats_t *out);

/* Copies the tree of the last make_tree to host arrays, for inspection and
 * parity tests.  perm[n_blobs] receives the original blob index of each
 * position in tree order.  Cell arrays (cap entries each; pass cap=0 to
 * query the count) describe the non-empty cells below the root in
 * depth-first pre-order, quadrants 0..3: level, [begin,end) in tree order,
 * leaf flag, centre and side length, and the nterms complex coefficients
 * (re,im interleaved) after M2M.  Returns the number of cells, or -1. */
long long tree2d_export_tree(int *perm, long long cap, int *level, int *begin, int *end, int *leaf,
                             double *cx, double *cy, double *region, double *coef);

/* FP64 direct O(N*M) sum of the regularised kernel (the yardstick of the
 * approximate modes): targets and sources in device memory. */
int tree2d_direct_device(int ntgt, const double *d_txy, int nsrc, const double *d_sxy,
                         const double *d_cir, const double *d_cor, double *d_uv, void *stream);

/* Near-field kernel tuning of the mixed/learned forms.  The variants give
 * bit-identical results and differ only in speed: source blobs read from
 * global memory (0: 4 warps per block, 1: 8) or staged in shared memory by
 * bulk copies (2: 4 warps, 3: 8, 4: 4 warps with more registers per thread,
 * fewer resident warps and a deeper unrolled pair loop).  autotune = 1
 * (default): the first solve of each (device, form, P, leaf-count class)
 * times every variant with CUDA events and keeps the fastest;
 * eval_variant >= 0 forces one (0 .. TREE2D_EVAL_VARIANTS - 1);
 * eval_variant = -1 with autotune = 0 runs variant 0.  No counterpart in
 * the reference. */
#define TREE2D_EVAL_VARIANTS 5

/* Mixed/learned forms with P = 16: on = 1 runs the M2M levels and the L2L
 * levels as one cooperative launch each, persistent blocks meeting at a
 * grid barrier between levels (bounded waits); on = 0 (default) launches
 * one kernel per level, which measured faster on GB300 (the barriers cost
 * more than the launches they save).  Results are the same either way.  No
 * counterpart in the reference. */
int tree2d_set_level_chain(int on);

/* Tile of the tensor-core M2L of the mixed/learned forms: cells per CTA.
 * rows = 128 gives each CTA a full 128-row MMA tile; rows = 64 fills half
 * of it (the other rows zero), so twice the CTAs share a level's cells,
 * which can hide more of the gather latency.  Results are bit-identical.
 * rows = 0 (default) lets the tuner pick on the first solve of each
 * (device, P, cell-count class), timing both with CUDA events (with
 * tree2d_set_tuning's autotune = 0: 128).  Other values:
 * TREE2D_ERR_BAD_PARAMS.  No counterpart in the reference. */
int tree2d_set_m2l_rows(int rows);
int tree2d_set_tuning(int autotune, int eval_variant);

/* Batched solve of nsets independent blob sets in one tree: set k is blobs
 * [set_offsets[k], set_offsets[k+1]) of the device arrays (set_offsets is a
 * host array of nsets + 1 ints, set_offsets[0] = 0, non-decreasing).  Each
 * set gets its own root box and exactly the cells, lists and cutoff it would
 * get alone, so every set's velocities equal those of solving it by itself;
 * the sets share every launch (one tree build, one pass of each expansion
 * kernel, one evaluation).  Mixed form only: TREE2D_ERR_MODE in the plain
 * mode or with a mirror wall (the learned mode runs the fixed mixed form
 * here).  No counterpart in the reference. */
int tree2d_solve_sets(int nsets, const int *set_offsets, const double *d_xy, const double *d_cir,
                      const double *d_cor, double *d_uv, void *stream);

/* Measures the FP64 FMA pipe: runs blocks x 256 threads x iters x 8
 * dependent-chain FMAs on `stream` and returns the elapsed device time in
 * milliseconds through *ms (flops = blocks*256*iters*16).  A measurement
 * helper for roofline reporting; no counterpart in the reference. */
int tree2d_fp64_probe(int blocks, int iters, void *stream, double *ms);
/* The same for bits = 64 (DFMA) or 32 (FFMA). */
int tree2d_pipe_probe(int bits, int blocks, int iters, void *stream, double *ms);
/* Failure-detection check of the bounded device waits: one kernel waits on
 * a shared-memory barrier that nothing completes, giving up after `polls`
 * polls exactly as the tensor-core kernels' waits do, and *status receives
 * TREE2D_ERR_TIMEOUT (what those kernels record when a wait gives up).
 * Returns TREE2D_OK when the probe itself ran.  No counterpart in the
 * reference. */
int tree2d_wait_probe(long long polls, int *status);

/* ------------------------------------------------------------------ */
/* Learned order selection (TREE2D_MODE_LEARNED).  A small network
 * (16 features -> 64 -> 64 -> 64 -> 14 classes, GELU, BF16 weights, FP32
 * accumulation) decides, for every near-field interaction of the mixed
 * form, between direct evaluation and the source leaf's multipole at order
 * p = 4..16.  Without weights the mode falls back to the fixed mixed form.
 * No counterpart in the reference. */

/* Number of network parameters (flat FP32 vector W1 b1 W2 b2 W3 b3 W4 b4). */
int tree2d_learn_param_count(void);
/* Loads a weights file (2dfmm_gb300/data/learned_weights.t2dw is the
 * packaged one): the parameters and the training envelope it records, as
 * tree2d_learn_set_weights + tree2d_learn_set_envelope do, so that a C or
 * Fortran caller enables TREE2D_MODE_LEARNED with one call.  Format,
 * little-endian: the bytes "T2DW", uint32 version (1), uint32 parameter
 * count, uint32 header size (32), float64 envelope limit (K-list source
 * blobs per leaf, 0 = none), float64 the correction radius it is counted at,
 * then the float32 parameters.  TREE2D_ERR_FILE for a missing or malformed
 * file (nothing is changed then). */
int tree2d_learn_load(const char *path);
int tree2d_learn_set_weights(const float *theta, int n);
int tree2d_learn_get_weights(float *theta, int n);
/* direct_bias: added to the direct-evaluation logit; order_margin: chosen
 * order raised by this much; budget: label tolerance per interaction in
 * units of sum|G| / root side.  Defaults 1.0, 1, 3e-7. */
int tree2d_learn_set_options(float direct_bias, int order_margin, double budget);
/* on = 1: the network also sets the expansion order of the far field's M2P
 * terms, each W-list entry (a cell's multipole evaluated at a leaf's blobs)
 * whose source is a leaf, presented to it as a U entry: the same order
 * classes and per-interaction budget; W entries with an internal-cell
 * source keep the full order.  on = 0 (default): every W entry at the full
 * order.  Off by default: with the packaged network it saved no time at
 * 4M two-patch + sheet blobs (7.43 against 7.41 ms per solve) and 0.4% at
 * 1M Lamb-Oseen blobs, and with it relL2 passes 1e-6 (packaged network:
 * 1.2e-6 at 262,144 two-patch + sheet blobs).  No counterpart in the
 * reference. */
int tree2d_learn_set_far_orders(int on);
/* Training envelope of the loaded network: the largest mean number of
 * source blobs in a leaf's K (correction) list leaves that the training
 * solves had, counted with the correction radius cutoff_sigmas (units of the
 * largest core radius; 0 = the radius in force).  A solve whose lists,
 * counted at that radius, hold more runs the fixed mixed form instead (the
 * network's per-interaction error budget does not bound the sum over more
 * interactions than it was trained on); tree2d_get_stats reports it in
 * learned_active and the solve's own figure in n_list_k_blobs.  Blobs, not
 * entries, make the figure independent of the leaf size.  When
 * cutoff_sigmas is above the radius in force, the list walk goes out to it
 * to count; below it, the blobs are counted at the radius in force (more of
 * them: the conservative side).  0 = no limit (the default). */
int tree2d_learn_set_envelope(double k_blobs_per_leaf_max, double cutoff_sigmas);
/* Training data from the last tree2d_solve_device in mixed or learned mode:
 * up to max_samples interactions drawn with `seed`, their features
 * (features[max][16]) and the cheapest class whose error against the FP64
 * exact contribution stays within the budget.  Returns the sample count,
 * or minus a status code (-TREE2D_ERR_MODE after a batched solve: samples
 * come from a solve of one set). */
int tree2d_learn_collect(int max_samples, unsigned seed, float *features, int *labels);
/* `steps` Adam steps on mini-batches of `batch` samples (host arrays),
 * starting from the loaded weights (or a seeded initialisation). */
int tree2d_learn_train(int n, const float *X, const int *y, int steps, int batch, float lr, unsigned seed,
                       float *loss);
/* Checking hooks: one forward + backward (mean cross-entropy) on n samples
 * with parameters theta, and the logits of n feature vectors by the
 * training path (CUDA cores, tensor_cores = 0) or the inference path
 * (tensor cores, 1).  Host arrays. */
int tree2d_mlp_grad(int n, const float *X, const int *y, const float *theta, float *grad, float *loss);
int tree2d_mlp_forward(int n, const float *X, const float *theta, float *logits, int tensor_cores);

/* Mirror wall at y = d_mirror (enable = 1): every solve adds the image of
 * each blob, (x, 2 d - y) with circulation -G as a point vortex (the
 * solver's image term, ver-c/src/includes/d_biot.f90:39-53), and returns the
 * velocities at the real blobs only.  The reference's tree path has no
 * mirror support (README: not supported); this is an extension. */
int tree2d_set_mirror(int enable, double d_mirror);

/* Device-resident time step: d_xy += dt * d_uv (forward Euler, the
 * solver's drift_b, e_drift.f90:17-59), on `stream`. */
int tree2d_advect_device(int n, double *d_xy, const double *d_uv, double dt, void *stream);

/* Library version string. */
const char *tree2d_version(void);

#ifdef __cplusplus
}
#endif
#endif
