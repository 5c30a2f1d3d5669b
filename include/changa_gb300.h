/*
 * Extension entry points of the GB300 gravity library.
 *
 * HostCUDA.h / EwaldCUDA.h carry the reference's FP32 boundary unchanged.
 * The forms below have no counterpart there; they take FP64 inputs that
 * live on the device and add:
 *   - the plain FP64 form (all arithmetic FP64),
 *   - the FP32-mixed form (positions split into a float high part and a
 *     float low part, the bucket-centre subtraction done in that split
 *     arithmetic, interactions in FP32, per-particle sums with Kahan
 *     compensation, FP64 results),
 *   - host helpers (Ewald h-table, request validation, error and completion
 *     plumbing).
 * All calls are asynchronous on the given stream and return 0 or a
 * CHANGA_E_* / cudaError_t code.
 *
 * Array layouts (row-major FP64):
 *   moments : 12 per node  {radius, soft, totalMass, cm.x, cm.y, cm.z,
 *             xx, xy, xz, yy, yz, zz}        (CudaMultipoleMoments order)
 *   parts   : 5 per particle {mass, soft, x, y, z} (CompactPartData order)
 *   vars    : 5 per particle {a.x, a.y, a.z, potential, dtGrav}; results
 *             accumulate (+=, max for dtGrav) like the reference kernels.
 */
#ifndef CHANGA_GB300_H_
#define CHANGA_GB300_H_

#include "HostCUDA.h"
#include "EwaldCUDA.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- errors, completion, validation ---- */

#define CHANGA_E_INVALID_ARG 1001   /* bad pointer / size / count */
#define CHANGA_E_INVALID_LIST 1002  /* list index or marker out of range */
#define CHANGA_E_TOO_LARGE 1003     /* size beyond a fixed limit */
#define CHANGA_E_DEVICE_WAIT 1004   /* a kernel's bounded wait ran out; its results are incomplete */

#define CHANGA_ERRORS_ABORT 0   /* print and abort() (reference behaviour) */
#define CHANGA_ERRORS_RECORD 1  /* record; read with changa_gb300_last_error */

void changa_gb300_set_error_mode(int mode);
/* Returns and clears the first error recorded since the last call (0: none). */
int changa_gb300_last_error(void);
const char *changa_gb300_error_string(int code);

/* Called by every drop-in entry point after its work is enqueued; the
 * stand-in for Charm++'s hapiAddCallback(stream, cb).  NULL (the default)
 * ignores cb. */
typedef void (*changa_completion_hook)(cudaStream_t stream, void *cb);
void changa_gb300_set_completion_hook(changa_completion_hook hook);

/* When on, the drop-in entry points check every list index, marker and
 * bucket range of a request on the host before any copy and reject a bad
 * request with CHANGA_E_INVALID_LIST (nothing is launched). */
void changa_gb300_set_validate(int on);

/* Host check of one request against its source and target array sizes. */
int changa_validate_request(const ILCell *list, long long n_entries, const int *markers,
                            const int *starts, const int *sizes, int n_buckets,
                            long long n_sources, long long n_targets);

int changa_gb300_version(void);

/* Measures the current device's FP32 FMA throughput (TFLOP/s, 2 FLOP per
 * fma.rn.f32, every SM busy): the roofline denominator of the list kernels,
 * whose bound is the FP32 FMA pipe.  Synchronous; allocates a small
 * buffer. */
int changa_gb300_fp32_fma_peak(double *tflops);

/* Number of kernels this library has launched since load (all forms). */
unsigned long long changa_gb300_kernel_launches(void);

/* Optional per-kernel timing: while on, every launch is bracketed by CUDA
 * events on its own stream.  changa_gb300_kernel_time() waits for and sums
 * the recorded launches of one kernel since its last read, then forgets
 * them.  Kernel ids: 0/1 drop-in FP32 cell/particle lists, 2/3 FP64,
 * 4/5 FP32-mixed, 6/7/8 Ewald FP32/FP64/mixed, 9 mixed-form packing,
 * 10/11 adjoint cell/particle lists, 12 moment up-pass and its adjoint. */
#define CHANGA_KERNEL_COUNT 13
void changa_gb300_set_timing(int on);
int changa_gb300_kernel_time(int kernel, double *total_ms, long long *launches);

/* Shape variants of the FP32-form list kernels (kernel ids 0, 1, 4, 5):
 * 0-4 source-parallel (resident blocks per SM x list chunks per reduction),
 * 5-7 target-parallel (2/3/4 blocks per SM), 8-10 target-parallel with
 * paired .f32x2 arithmetic (2/3/4 blocks per SM; defaults 8 for cell lists,
 * 10 for particle lists), 11-12 paired with the FP32-mixed cell records
 * staged by TMA tile::gather4 copies (2/1 blocks per SM; the other lists
 * run the paired kernel), 13-16 paired with 1-3 targets per lane chosen
 * per bucket (blocks per SM / most targets per lane: 2/3, 2/2, 3/2, 1/3),
 * which keeps the lanes of buckets of 17-31 targets busy.  The autotuner
 * (changa_gb300/autotune.py) times them on a workload and selects one per
 * kernel. */
int changa_gb300_list_variant_count(void);
int changa_gb300_set_list_variant(int kernel, int variant);
int changa_gb300_get_list_variant(int kernel);
/* The FP32-mixed hexadecapole cell kernel: 0 synchronous staging, 1 / 2
 * paired .f32x2 arithmetic with 1 / 2 resident blocks per SM (default 2). */
int changa_gb300_set_hex_variant(int variant);
int changa_gb300_get_hex_variant(void);

/* The TMA-staged variants (11-12) wait for their copies with an iteration
 * limit.  A wait that runs out marks the device's status word and ends that
 * warp's work, so some buckets' forces are incomplete.  This call waits for
 * the current device, then reads and clears the word: it returns 0, or
 * CHANGA_E_DEVICE_WAIT (recorded like any other error) when a wait ran out
 * since the last read.  changa_gravity_step_host reads the word itself when
 * it launched a TMA variant.  Kernels that finish while this call reads
 * are seen by the next call. */
int changa_gb300_device_status(void);
/* Test hook: the poll limit of those waits (a negative value restores the
 * default, 2^22).  0 makes every wait run out at once, on purpose; the copy
 * in flight is still waited for (with a long limit) before the warp stops. */
void changa_gb300_set_test_wait_limit(int polls);

/* ---- device-resident list requests for the extension forms ---- */

typedef struct ChangaListRequest {
  const ILCell *list;   /* device: entries, ILCell {index, offsetID} */
  const int *markers;   /* device: n_buckets + 1 CSR offsets into list */
  const int *starts;    /* device: first target of each bucket */
  const int *sizes;     /* device: targets in each bucket */
  int n_buckets;
  long long n_entries;
} ChangaListRequest;

/* Plain FP64 form: cell lists (nodeBucketForce) / particle lists
 * (partBucketForce) over FP64 arrays. */
int changa_cell_forces_fp64(const double *moments, long long n_moments,
                            const double *targets, long long n_targets,
                            const ChangaListRequest *req, double fperiod, double *vars,
                            cudaStream_t stream);
int changa_part_forces_fp64(const double *sources, long long n_sources,
                            const double *targets, long long n_targets,
                            const ChangaListRequest *req, double fperiod, double *vars,
                            cudaStream_t stream);

/* FP32-mixed form of the same two evaluations. */
int changa_cell_forces_mixed(const double *moments, long long n_moments,
                             const double *targets, long long n_targets,
                             const ChangaListRequest *req, double fperiod, double *vars,
                             cudaStream_t stream);
int changa_part_forces_mixed(const double *sources, long long n_sources,
                             const double *targets, long long n_targets,
                             const ChangaListRequest *req, double fperiod, double *vars,
                             cudaStream_t stream);

/* changa_cell_forces_mixed without any device allocation.  No counterpart
 * in the reference.  For callers that must not let a library allocate (a
 * host code whose device memory is all handed to its own pool allocator, or
 * one that enqueues from a thread that must never wait for the device, as
 * cudaMalloc/cudaFree can synchronise it).  The scratch (packed moments,
 * packed targets, work-queue counter) lives in one fixed 16 MiB + 256 B
 * array inside the library, held on every GPU that loads it until exit;
 * 64 B x n_moments + 32 B x n_targets must fit in 16 MiB (each rounded up to
 * 256 B), else CHANGA_E_TOO_LARGE and nothing is enqueued.  The first call
 * on a device looks up the array's device address: make it before any
 * stream capture.  The address is cached per device and context id, so the
 * first call after a cudaDeviceReset looks it up again (make that call
 * before any capture too).  Calls share the array: two calls that overlap on the GPU
 * race; order them on one stream.  Inputs and outputs as for
 * changa_cell_forces_mixed (device pointers). */
int changa_cell_forces_mixed_noalloc(const double *moments, long long n_moments,
                                     const double *targets, long long n_targets,
                                     const ChangaListRequest *req, double fperiod,
                                     double *vars, cudaStream_t stream);

/* One whole force evaluation: cell lists + particle lists (+ Ewald when
 * ewald != NULL) for particles that are both sources and targets.
 * form: CHANGA_FORM_FP64 or CHANGA_FORM_MIXED. */
#define CHANGA_FORM_FP32 0
#define CHANGA_FORM_FP64 1
#define CHANGA_FORM_MIXED 2

typedef struct ChangaEwaldParams {
  double root[12];   /* root moments, moments layout */
  double L;          /* period */
  int nReps;         /* replicas the walk covered (the erf hole) */
  double fEwCut;     /* real-space cut in periods */
  int nEwhLoop;      /* rows in ewt, at most CHANGA_MAX_EWH */
  const double *ewt; /* HOST: nEwhLoop x 5 {hx, hy, hz, hCfac, hSfac} */
  const double *momc; /* HOST: the root's complete moments (MomcData order,
                         32 values, changa_ewald_table_hex); read only by
                         changa_gravity_step_hexa, which then takes M and cm
                         from root[2..5] */
} ChangaEwaldParams;

#define CHANGA_MAX_EWH 256

int changa_gravity_step(int form, const double *moments, long long n_moments,
                        const double *parts, long long n_parts,
                        const ChangaListRequest *cells, const ChangaListRequest *plist,
                        double fperiod, const ChangaEwaldParams *ewald,
                        double *vars, cudaStream_t stream);

/* The same evaluation from HOST arrays: the requests' pointers, moments,
 * parts and the ewt table are host memory (pinned memory copies fastest).
 * The interaction lists are uploaded in chunks on a library-owned copy
 * stream while the list kernels run on `stream` over the chunks already
 * landed.  Results ACCUMULATE into vars (host, n_parts x 5); with
 * form | CHANGA_STEP_OVERWRITE they replace it instead (vars is not read,
 * so a fresh evaluation needs no zeroed host buffer).  When vars is pinned
 * and the last list's chunks write disjoint particle ranges, each range is
 * read back on a second copy stream as soon as its kernel is done.
 * Returns after the work has finished, so vars is ready on return. */
#define CHANGA_STEP_OVERWRITE 0x100

/* Particle lists as runs of consecutive source particles, one ILPart
 * {first source particle, offsetID, num} per run: the form ChaNGa's walk
 * produces (a source bucket is one run) before the reference flattens it to
 * one ILCell per particle.  All host arrays.  Bucket b owns runs
 * [run_markers[b], run_markers[b+1]) and, once expanded, the flat entries
 * [markers[b], markers[b+1]) (so markers[b+1] - markers[b] is the sum of its
 * runs' num); starts and sizes as in ChangaListRequest. */
typedef struct ChangaPartRuns {
  const ILPart *runs;
  const int *run_markers;  /* n_buckets + 1 */
  const int *markers;      /* n_buckets + 1 */
  const int *starts;
  const int *sizes;
  int n_buckets;
  long long n_runs;
} ChangaPartRuns;

/* changa_gravity_step_host with the particle lists as runs: each chunk of
 * runs is uploaded (12 bytes per run instead of 8 per source particle),
 * expanded into flat entries on the device and evaluated as it lands.  The
 * same results as the flat lists. */
int changa_gravity_step_host_runs(int form, const double *moments, long long n_moments,
                                  const double *parts, long long n_parts,
                                  const ChangaListRequest *cells, const ChangaPartRuns *pruns,
                                  double fperiod, const ChangaEwaldParams *ewald, double *vars,
                                  cudaStream_t stream);

/* List bytes per upload chunk of changa_gravity_step_host and of the
 * drop-in list transfers (default 256 MiB, at least 4 KiB; 0 restores the
 * default).  changa_gravity_step_host uploads the particles first, in
 * slices of a quarter chunk.  A drop-in
 * request whose list exceeds two chunks uploads it chunk by chunk on the
 * library's copy stream, each chunk's buckets evaluated as it lands. */
void changa_gb300_set_host_chunk_bytes(size_t bytes);
int changa_gravity_step_host(int form, const double *moments, long long n_moments,
                             const double *parts, long long n_parts,
                             const ChangaListRequest *cells, const ChangaListRequest *plist,
                             double fperiod, const ChangaEwaldParams *ewald,
                             double *vars, cudaStream_t stream);

/* changa_gravity_step captured once into a CUDA graph and replayed: the
 * batching form.  The requests may span many independent systems
 * concatenated (indices and starts shifted); the persistent list kernels'
 * device work queue balances their uneven buckets inside one replay.  The
 * graph keeps the device pointers it was created with: update the arrays in
 * place between launches.  The ChangaEwaldParams and requests are read at
 * creation only.  Returns NULL on error (see changa_gb300_last_error). */
typedef struct ChangaGravityGraph ChangaGravityGraph;
ChangaGravityGraph *changa_gravity_graph_create(int form, const double *moments,
                                                long long n_moments, const double *parts,
                                                long long n_parts,
                                                const ChangaListRequest *cells,
                                                const ChangaListRequest *plist, double fperiod,
                                                const ChangaEwaldParams *ewald, double *vars,
                                                int zero_vars);
int changa_gravity_graph_launch(ChangaGravityGraph *g, cudaStream_t stream);
void changa_gravity_graph_destroy(ChangaGravityGraph *g);

/* Hexadecapole build (ChaNGa's default configuration, HEXADECAPOLE): one
 * evaluation with cells in the 27-double hexadecapole layout {radius, soft,
 * totalMass, cm.xyz, xx xy xz yy yz, xxx xyy xxy yyy xxz yyz xyz, xxxx xyyy
 * xxxy yyyy xxxz yyyz xxyy xxyz xyyz} (moments scaled by the radius,
 * reduced: cuda_typedef.h:103-128, moments.h FMOMR), evaluated by
 * momEvalFmomrcm (gravity.h:439-446) from `cells`; `softcells` lists the
 * cells whose softening meets the bucket, evaluated as softened point
 * masses {M, soft, cm} (gravity.h:414-421); `plist` as in
 * changa_gravity_step.  form: CHANGA_FORM_FP64 or CHANGA_FORM_MIXED;
 * isolated or periodic lists (fperiod).  ewald (may be NULL): the
 * hexadecapole Ewald correction (BucketEwald with HEXADECAPOLE,
 * Ewald.cpp:72-281) about the root with complete moments ewald->momc and
 * the table of changa_ewald_table_hex. */
int changa_gravity_step_hexa(int form, const double *moments, long long n_moments,
                             const double *parts, long long n_parts,
                             const ChangaListRequest *cells, const ChangaListRequest *plist,
                             const ChangaListRequest *softcells, double fperiod,
                             const ChangaEwaldParams *ewald, double *vars, cudaStream_t stream);

/* Adjoint of the cell + particle list accelerations (FP32-mixed; no
 * reference counterpart): given lam = dL/da (n_parts x 3), ACCUMULATES
 * dL/dx and dL/dm into grad (n_parts x 4 {dx, dy, dz, dm}) through the same
 * lists, the tidal tensor of every interaction and the moment construction
 * (tree topology held fixed).  parent: BFS parent of every moment (-1 at
 * the root); leaf: moment index of each particle's bucket.  fperiod: the
 * period of the lists' replica offsets (0 for isolated systems); the
 * Ewald term's part is changa_ewald_vjp. */
int changa_gravity_vjp_mixed(const double *moments, long long n_moments, const double *parts,
                             long long n_parts, const ChangaListRequest *cells,
                             const ChangaListRequest *plist, double fperiod, const int *parent,
                             const int *leaf, const double *lam, double *grad,
                             cudaStream_t stream);

/* Adjoint of the Ewald term of the quadrupole build (FP64; no reference
 * counterpart): given lam = dL/da (n_parts x 3, the particles' order in
 * parts), ACCUMULATES into grad (n_parts x 4 {dx, dy, dz, dm}) the
 * derivative of sum lam . a_ewald, both through each particle's own position
 * (the tidal tensor of the real-space replica terms and of the Fourier
 * sum) and through the root moments (mass, centre of mass, quadrupole) that
 * every particle shapes.  p: the parameters the forward evaluation used
 * (root moments and h-table of changa_ewald_table).  Together with
 * changa_gravity_vjp_mixed at fperiod it gives the adjoint of a periodic
 * evaluation.  CHANGA_E_INVALID_ARG for a root without mass or a table
 * with sine terms (the hexadecapole build's). */
int changa_ewald_vjp(const double *parts, long long n_parts, const ChangaEwaldParams *p,
                     const double *lam, double *grad, cudaStream_t stream);

/* Moment up-pass on the device over a fixed topology (no reference
 * counterpart; the reference builds moments on the host,
 * MultipoleMoments.h:206-352): for every moment i, recomputes soft,
 * totalMass, cm and xx..zz of moments[i] (FP64, moments layout) from the
 * particles parts[first[i] .. first[i] + count[i]) (parts layout, GPU
 * order); the radius is kept.  first/count: device int arrays. */
int changa_tree_moments(const double *parts, long long n_parts, const int *first,
                        const int *count, long long n_moments, double *moments,
                        cudaStream_t stream);

/* Direct-sum accuracy yardstick (no reference counterpart): the force on
 * the particles parts[idx[k]] from every particle, without a tree.  L == 0:
 * open boundaries, SPLINE softening, out[k] = {ax, ay, az, pot}.  L > 0:
 * periodic cube of side L by Ewald summation (real space within
 * rcut_frac * L of the minimum image, 0 < rcut_frac <= 0.5, 0 selects 0.5;
 * k space to exp(-k^2 / 4 alpha^2) = 1e-9), out[k] = {ax, ay, az, 0}.
 * Pair terms in FP32 on split coordinates with compensated sums, S(k) and
 * totals in FP64: about 1e-6 of |a|.  parts: device FP64 (parts layout);
 * idx: device int; out: device FP64 n_idx x 4 (overwritten).  Returns after
 * the stream has finished. */
int changa_direct_forces(const double *parts, long long n_parts, const int *idx, long long n_idx,
                         double L, double rcut_frac, double *out, cudaStream_t stream);

/* Interaction-list walk on the device (no reference counterpart in the
 * default build; the reference's GPU walk prototype is gpuLocalTreeWalk,
 * HostCUDA.cu:724-942).  One thread per target bucket reproduces the host
 * dual walk's per-bucket lists (the same entries, in depth-first order).
 * Tree arrays in moment (breadth-first) order, device memory:
 *   geom   n_nodes x 6 {cm.xyz, radius, soft, mass}
 *   bbox   n_nodes x 6 {lesser xyz, greater xyz} of the node's particles
 *   info   n_nodes x 4 {child0, child1, first, count} (-1: no child)
 *   parent n_nodes (-1 at the root); bucket_node: moment index per bucket. */
typedef struct ChangaTreeView {
  const double *geom;
  const double *bbox;
  const int *info;
  const int *parent;
  long long n_nodes;
  const int *bucket_node;
  int n_buckets;
} ChangaTreeView;

typedef struct ChangaWalkParams {
  double theta;   /* opening angle; the hexadecapole monopole angle is theta^4 */
  int order;      /* 2 quadrupole, 4 hexadecapole (adds the softened-cell list) */
  double period;  /* 0 for open boundaries */
  int n_replicas; /* replica layers on the root check list (0..3) */
} ChangaWalkParams;

/* Count pass: per-bucket list lengths (device int arrays, n_buckets each;
 * n_soft only for order 4).  Returns after the stream has finished. */
int changa_walk_count(const ChangaTreeView *tree, const ChangaWalkParams *p, int *n_cells,
                      int *n_parts, int *n_soft, cudaStream_t stream);
/* Fill pass: writes each bucket's entries at its offset (device long long
 * arrays, exclusive prefix sums of the counts) into the device lists.
 * Cells and softened cells index the moments, particles index the parts;
 * offsetID = replica code << 22.  Returns after the stream has finished. */
int changa_walk_fill(const ChangaTreeView *tree, const ChangaWalkParams *p,
                     const long long *off_cells, const long long *off_parts,
                     const long long *off_soft, ILCell *cells, ILCell *parts, ILCell *soft,
                     cudaStream_t stream);

/* The whole walk in one call.  Trees of 16384 buckets or more take one
 * traversal: a count of every 16th bucket sizes pools of 256-entry chunks,
 * one pass counts every bucket's lists and appends their entries chunk by
 * chunk, and a gather puts the chunks in list order (a fill pass replaces
 * the gather if a pool ran short).  Smaller trees count, then fill.  The
 * lists and markers are device arrays owned by the result until
 * changa_walk_lists_free: list k (0 cells, 1 particles, 2 softened cells
 * when order is 4) holds n_entries[k] ILCells, bucket b's entries at
 * markers[k][b] .. markers[k][b + 1], in the same order as count + fill
 * write them.  passes: 1 (append + gather), 2 (count + fill), 3 (append,
 * then fill).  Returns after the stream has finished. */
typedef struct ChangaWalkLists {
  int n_buckets;
  int order;
  int passes;
  long long n_entries[3];
  ILCell *list[3];
  int *markers[3];
} ChangaWalkLists;
int changa_walk(const ChangaTreeView *tree, const ChangaWalkParams *p, ChangaWalkLists *out,
                cudaStream_t stream);
void changa_walk_lists_free(ChangaWalkLists *out);
/* Append-pass pool capacity as a multiple of the sampled estimate of the
 * entries (default 1.2; 0 leaves one chunk per bucket and list, so lists
 * longer than one chunk end in the fill pass). */
void changa_walk_set_pool_factor(double factor);
/* Testing only: with on != 0, each traversal first runs with a 64-entry
 * stack per warp, so that the re-run with the large stack (taken when a
 * warp exhausts its stack) is exercised. */
void changa_walk_set_test_small_stack(int on);
/* Traversal launches re-run with the large stack so far (in this process). */
long long changa_walk_stack_reruns(void);
/* changa_walk of a tree with at least min_tree_buckets buckets walks in
 * two phases: first once per group of at most max_buckets buckets
 * (the highest node whose subtree holds no more), down to the group node,
 * which the group's buckets share; then each bucket from the entries still
 * undecided there.  The lists hold the same entries as the one-phase walk.
 * Defaults 32 and 4096; 0 for either walks every bucket from the root. */
void changa_walk_set_groups(int max_buckets, int min_tree_buckets);

/* Walk and forces in one pass, with no interaction lists (FP32-mixed form,
 * quadrupole trees).  Phase 1 of the two-phase walk writes each group's
 * prefix lists and frontier; then a warp per bucket walks from its group's
 * frontier and evaluates each 32 accepted cells or opened particles as they
 * are decided, with the list kernels' paired arithmetic (the reference's
 * prototype of the idea: gpuLocalTreeWalk, HostCUDA.cu:724-942).
 * moments: n_nodes x 12 FP64 in the tree's node order (the moments the list
 * entries index), parts: n_parts x 5 {m, soft, x, y, z} in tree order,
 * vars: n_parts x 5 FP64, WRITTEN (not accumulated) for every particle of a
 * bucket, then the Ewald term added when ewald is given.  The interactions
 * are the list walk's; the sums agree with changa_gravity_step on its lists
 * to FP32 summation order.  On GB300 it is slower than changa_walk plus
 * changa_gravity_step (nfw8m: 86.6 ms against 37.7 ms), which stays the
 * fast route.  Returns after the stream has finished. */
int changa_walk_forces(const ChangaTreeView *tree, const ChangaWalkParams *p,
                       const double *moments, const double *parts, long long n_parts,
                       const ChangaEwaldParams *ewald, double *vars, cudaStream_t stream);

/* Tree build on the device (no reference counterpart; restates the host
 * build, TreePiece.cpp:141-165 box and keys, GenericTreeNode.h:473-599
 * split, MultipoleMoments.h:206-352, 460-526 moments and radii): positions
 * (n x 3), masses and softenings are device FP64 arrays.  The handle owns
 * the device arrays below until changa_tree_free; NULL on error. */
typedef struct ChangaTree ChangaTree;
typedef struct ChangaTreeArrays {
  long long n, n_nodes;
  int n_buckets;
  const int *perm;        /* n: GPU (key) order -> input index */
  const double *parts;    /* n x 5, GPU order */
  const double *moments;  /* n_nodes x 12, breadth-first */
  const double *geom;     /* n_nodes x 6 {cm.xyz, radius, soft, mass} */
  const double *bbox;     /* n_nodes x 6 */
  const int *info;        /* n_nodes x 4 {child0, child1, first, count} */
  const int *parent;      /* n_nodes, -1 at the root */
  const int *bucket_node; /* n_buckets, key order */
  const int *leaf;        /* n: bucket node of each particle */
  const double *box;      /* 6: the cubical bounding box */
} ChangaTreeArrays;
ChangaTree *changa_tree_build(const double *pos, const double *mass, const double *soft,
                              long long n, int n_bucket, cudaStream_t stream);
int changa_tree_view(const ChangaTree *tree, ChangaTreeArrays *out);
void changa_tree_free(ChangaTree *tree);

/* Ewald correction for parts[idx[k]] into vars[idx[k]] (idx == NULL: the
 * first n_idx particles).  form: FP64 or MIXED. */
int changa_ewald_forces(int form, const double *parts, long long n_parts, const int *idx,
                        long long n_idx, const ChangaEwaldParams *p, double *vars,
                        cudaStream_t stream);

/* Host restatement of TreePiece::EwaldInit (Ewald.cpp:285-383): fills up to
 * max_h rows of ewt; returns nEwhLoop, or -1 if max_h is too small. */
int changa_ewald_table(const double *root, double L, double dEwhCut, double *ewt, int max_h);
/* The hexadecapole build's table (TreePiece::EwaldInit with HEXADECAPOLE,
 * Ewald.cpp:285-383): root holds the 27 hexadecapole moment values
 * {radius, soft, M, cm, 21 scaled reduced moments}; the rows are as above
 * (hSfac now carries the octupole).  momc, if not NULL, receives the root's
 * complete moments in MomcData order (32 doubles), the values
 * EwaldReadOnlyData.momcRoot carries in that build. */
int changa_ewald_table_hex(const double *root, double L, double dEwhCut, double *ewt,
                           int max_h, double *momc);

#ifdef __cplusplus
}
#endif

#endif /* CHANGA_GB300_H_ */
