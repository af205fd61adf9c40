/*
 * librett_c.h -- C-ABI (extern "C") surface of the GB300 tensor-transpose
 * engine, for FFI callers (ctypes, cffi, cgo, JNI ...).  Plain pointers and
 * sizes only; the stream is an opaque `void*` holding a cudaStream_t (NULL is
 * the legacy default stream).  Every function returns a librettResult value
 * (0 = LIBRETT_SUCCESS) as an int.
 *
 * Each entry point is a thin wrapper over the C++ interface in librett.h,
 * which mirrors LibreTT's src/librett.h; the citation on each line names the
 * LibreTT declaration it replaces.
 */
#ifndef LIBRETT_C_H
#define LIBRETT_C_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifndef LIBRETT_H
typedef unsigned int librettHandle;
#endif

/* Transpose methods; numbering follows LibreTT src/plan.h:54-56. */
enum {
  LIBRETT_METHOD_UNKNOWN = 0,
  LIBRETT_METHOD_TRIVIAL = 1,      /* fused rank 1: plain copy                    */
  LIBRETT_METHOD_PACKED = 2,       /* whole Mm u Mk sub-volume per tile           */
  LIBRETT_METHOD_PACKED_SPLIT = 3, /* as Packed with one rank cut into chunks     */
  LIBRETT_METHOD_TILED = 4,        /* 2-rank tile of (in rank 0) x (out rank 0)   */
  LIBRETT_METHOD_TILED_COPY = 5    /* leading rank shared: strided row copy       */
};

/* Description of a plan: what the planner chose and why. */
typedef struct librett_plan_info {
  int method;                      /* LIBRETT_METHOD_*                            */
  int element_bytes;               /* sizeofType                                  */
  int fused_rank;                  /* rank after dropping unit dims and fusing    */
  int fused_perm[16];              /* permutation of the fused problem            */
  long long fused_dim[16];         /* dims of the fused problem (input order)     */
  long long tile_extent[16];       /* per fused rank: extent covered by one tile  */
  long long volume;                /* elements                                    */
  long long num_tiles;             /* tiles (or rows / chunks) per launch         */
  int threads;                     /* threads per CTA                             */
  int slots;                       /* elements (or units) per thread per tile     */
  int smem_bytes;                  /* dynamic shared memory per CTA               */
  int pad_shift;                   /* smem padding: 1 element per 2^pad_shift    */
  int pipeline;                    /* tile: 0 register-staged, 1 cp.async ring,
                                      2 one tile per CTA, 3 the same with bulk
                                      copies (cp.async.bulk + mbarrier)        */
  int unit_in_bytes;               /* global load width                           */
  int unit_out_bytes;              /* global store width                          */
  int run_in_bytes;                /* contiguous input run per tile               */
  int run_out_bytes;               /* contiguous output run per tile              */
  int grid;                        /* CTAs launched (0 if not yet known)          */
  int candidate;                   /* index into the planner's candidate list     */
  int num_candidates;              /* candidates the planner enumerated           */
  double model_cost;               /* analytic cost estimate (seconds)            */
  int selected_by;                 /* 0 analytic model, 1 learned model,
                                      2 measurement, 3 explicit candidate         */
  int table_bytes;                 /* device offset tables the plan holds: 0 for
                                      tiles of at most 6 ranks (addresses
                                      computed in the kernel) and non-tile plans */
} librett_plan_info;

/* librettInitialize / librettFinalize (LibreTT src/librett.h:57,62). */
void librett_c_initialize(void);
void librett_c_finalize(void);

/* librettPlan (LibreTT src/librett.h:78). */
int librett_c_plan(librettHandle* handle, int rank, const int* dim, const int* permutation,
                   size_t sizeofType, void* stream);

/* librettPlanMeasure (LibreTT src/librett.h:96-97). Overwrites odata. */
int librett_c_plan_measure(librettHandle* handle, int rank, const int* dim,
                           const int* permutation, size_t sizeofType, void* stream,
                           const void* idata, void* odata);

/* librettExecute (LibreTT src/librett.h:121). Asynchronous on the plan's stream. */
int librett_c_execute(librettHandle handle, const void* idata, void* odata);

/* librettDestroy (LibreTT src/librett.h:108). */
int librett_c_destroy(librettHandle handle);

/* Plan introspection; no LibreTT counterpart (LibreTT prints it with
 * librettPlan_t::print, src/plan.cpp:825-833). */
int librett_c_plan_info(librettHandle handle, librett_plan_info* info);

/* Device status of a plan, read after the plan's stream has drained
 * (synchronises it): 0, or 1 when a launch of the bulk-copy pipeline
 * (pipeline 3) waited longer than its limit for its copies and skipped its
 * stores.  The plan's word is one of 65,536 shared device words that a
 * timed-out launch tags with its plan; a later timeout of another plan on
 * the same word (plans created 65,536 apart) overwrites it.  Plans of other
 * pipelines always read 0.  No LibreTT counterpart (LibreTT exits on device
 * errors, src/GpuUtils.h:47-56). */
int librett_c_plan_status(librettHandle handle, unsigned* status);

/* Test hook for the bulk-copy pipeline's bounded wait (no LibreTT
 * counterpart): launches the plan (which must be a bulk-copy plan, pointers
 * 16-byte aligned) once with `extra_bytes` (1..4096) more transaction bytes
 * armed on each CTA's mbarrier than its copies deliver, so that no wait can
 * complete: every CTA gives up after its time limit (about 1 s, then up to
 * 1 s more for its copies), tags the plan's status word and skips its
 * stores.  Synchronises the plan's stream, returns the plan's status after
 * the launch in *status (1 expected, as librett_c_plan_status) and clears
 * it; the plan stays usable.  Nothing faults: the copies complete, only the
 * armed count is never reached. */
int librett_c_bulk_wait_test(librettHandle handle, const void* idata, void* odata,
                             unsigned extra_bytes, unsigned* status);

/* Host-only planning without a device or a handle: runs the same input check,
 * rank fusion and tile choice as librett_c_plan for a device with `num_sms`
 * SMs.  candidate < 0 picks the planner's default; otherwise the numbered
 * candidate.  No LibreTT counterpart (used by tests and tools). */
int librett_c_describe(int rank, const int* dim, const int* permutation, size_t sizeofType,
                       int num_sms, int candidate, librett_plan_info* info);

/* Create a plan using a specific candidate (index as in librett_plan_info).
 * No LibreTT counterpart; used by autotuning and by plan-choice studies. */
int librett_c_plan_candidate(librettHandle* handle, int rank, const int* dim,
                             const int* permutation, size_t sizeofType, void* stream,
                             int candidate);

/* Transpose in one call without allocating device memory; no counterpart in
 * LibreTT.  For callers that may not allocate device memory while running
 * (device memory reserved up front by their own allocator, or allocation
 * forbidden on a latency-critical path); librett_c_plan may allocate the
 * offset tables of its plan, this call does not.  It plans on the host,
 * writes the tile's offset tables into one fixed 64 KiB device array that
 * the library holds on every GPU that loads it, and launches on `stream`.
 * Returns LIBRETT_INVALID_PARAMETER if a tile's tables would exceed the
 * array (cannot happen for tiles this planner makes).  The first call on a
 * device looks up the array's address on that device: make it before any
 * stream capture.  All calls share the array and every call rewrites the
 * part it reads, so nothing needs to start at zero; calls that can overlap
 * on the GPU (other streams, other host threads) race on it and must be
 * ordered by the caller.  Inputs and outputs as for librett_c_execute. */
int librett_c_transpose_noalloc(int rank, const int* dim, const int* permutation,
                                size_t sizeofType, void* stream, const void* idata,
                                void* odata);

/* Device-side verifier (the role of LibreTT's device checker,
 * src/TensorTester.cpp:47-126): compares every element of odata with the
 * element of idata the transpose formula names, on the device, and returns
 * the number of mismatching elements and the smallest mismatching output
 * index (-1 if none).  Synchronises `stream`. */
int librett_c_verify(int rank, const int* dim, const int* permutation, size_t sizeofType,
                     const void* idata, const void* odata, void* stream,
                     unsigned long long* mismatches, long long* first_bad);

/* ---- Learned plan selection (no LibreTT counterpart; replaces the role of
 * LibreTT's analytic GpuModel ranking, src/plan.cpp:1073-1643) ---- */

/* Feature vector (nfeatures >= librett_c_mlp_feature_count()) of one
 * candidate, host-only. */
int librett_c_candidate_features(int rank, const int* dim, const int* permutation,
                                 size_t sizeofType, int num_sms, int candidate, float* features,
                                 int nfeatures);

/* Which model ranks candidates: 0 learned when a model for this device is
 * loaded else analytic (default), 1 analytic, 2 learned.  Returns the
 * previous mode, or -1 for an invalid mode.  The LIBRETT_PLAN_SELECTOR
 * environment variable (auto / analytic / learned) sets the initial mode. */
int librett_c_set_plan_selector(int mode);

/* Candidate set: 0 (default) tile plans in the one-tile-per-CTA pipeline
 * only; 1 also the persistent register-staged and cp.async pipelines (the
 * LIBRETT_ALL_PIPELINES=1 environment variable sets 1).  Returns the
 * previous setting.  Changes candidate numbering. */
int librett_c_set_candidate_set(int all);

/* Plan cache (no LibreTT counterpart): librett_c_plan / librettPlan reuse
 * the planner's choice for a fused problem already planned on this device.
 * Sets the capacity in entries (0 disables; the LIBRETT_PLAN_CACHE
 * environment variable sets the initial value, default 4096) and returns the
 * previous one.  Changing the selector, its model or the candidate set
 * clears the cache. */
int librett_c_set_plan_cache(int capacity);
int librett_c_plan_cache_stats(long long* hits, long long* misses, int* entries);

/* Load a weight file (NULL: the default, LIBRETT_PLAN_MODEL or
 * models/plan_mlp.bin next to the library).  A missing, truncated,
 * corrupt or non-finite file is rejected and the analytic model stays in
 * use. */
int librett_c_load_plan_model(const char* path);

/* MLP sizes and device-pointer kernels used to train the selector on the
 * GPU (forward with saved activations, backward, MSE gradient, Adam). */
int librett_c_mlp_param_count(void);
int librett_c_mlp_feature_count(void);
int librett_c_mlp_workspace_floats(int batch);
int librett_c_mlp_forward(const float* params, const float* X, int batch, float* ws, float* out,
                          void* stream);
int librett_c_mlp_backward(const float* params, const float* X, int batch, float* ws,
                           const float* dout, float* grads, void* stream);
int librett_c_mlp_mse_grad(const float* out, const float* y, int batch, float* dout, float* loss,
                           void* stream);
int librett_c_mlp_adam(float* params, const float* grads, float* m, float* v, int n, float lr,
                       float beta1, float beta2, float eps, int step, void* stream);

/* Host forward pass (standardised inputs, n rows of features) -- the
 * inference librettPlan runs. */
int librett_c_mlp_predict_host(const float* params, const float* x, int n, float* out);

/* ---- Grouped execution (no LibreTT counterpart; see librett.h) ---- */
#ifndef LIBRETT_H
typedef unsigned int librettGroupHandle;
#endif
int librett_c_group_create(librettGroupHandle* group, int count, const librettHandle* plans,
                           void* const* idata, void* const* odata, void* stream);
/* As librett_c_group_create with the policy given per member class
 * (policy[12]: class = size class + 4 * element-size index; size classes
 * < 64 KiB, < 1 MiB, < 16 MiB, larger; element sizes 4, 8, 16).  A policy is
 * tile + 4 * loads: tile 0 = plan selector's tile, 1 = largest tile within
 * 10% of the best sector efficiency, 2 = largest tile, 3 = analytic model for
 * a full device; loads 0 = through registers, 1 = cp.async into shared
 * memory (one tile per CTA), 2 = cp.async with persistent CTAs (one wave of
 * SMs x occupancy walking the bucket's tiles).  Values 0..11. */
int librett_c_group_create_policy(librettGroupHandle* group, int count,
                                  const librettHandle* plans, void* const* idata,
                                  void* const* odata, void* stream, const int* policy);
int librett_c_group_tune(librettGroupHandle group);
/* Bucket `index` (launch order) of the group's graph: shape[6] = element
 * bytes, load unit, store unit (elements), load units per thread, dynamic
 * shared memory bytes, loads (0/1/2 as in the policy); its members, tiles
 * and algorithmic bytes. */
int librett_c_group_bucket(librettGroupHandle group, int index, int* shape, int* members,
                           long long* tiles, long long* bytes);
/* policy[12] in use, and whether it came from tuning (this group's or a
 * cached one for the same batch signature). */
int librett_c_group_policy(librettGroupHandle group, int* policy, int* tuned);
int librett_c_group_execute(librettGroupHandle group);
int librett_c_group_destroy(librettGroupHandle group);
int librett_c_execute_grouped(int count, const librettHandle* plans, void* const* idata,
                              void* const* odata);
/* Host-only self-check of grouped execution's run tables for flat-tile
 * candidate `candidate` (in element units when element_units != 0): the
 * kernel's run-split index arithmetic must reproduce the per-unit offset
 * tables of the single-plan kernel for every unit of the tile.  Returns
 * LIBRETT_SUCCESS when it does, LIBRETT_INTERNAL_ERROR on a mismatch,
 * LIBRETT_INVALID_DEVICE when the tile's vector units cross a run (the group
 * then moves that member in element units), LIBRETT_INVALID_PARAMETER for a
 * bad problem or candidate. */
int librett_c_group_run_check(int rank, const int* dim, const int* permutation, size_t sizeofType,
                              int num_sms, int candidate, int element_units);

/* Host-only self-check of the bulk-copy pipeline for candidate `candidate`
 * of the planner's candidate list (candidate set 1): every segment the
 * kernel copies with one cp.async.bulk must be contiguous in global memory
 * (per the load-unit table) and in shared memory (between padding gaps),
 * 16-byte aligned in both, and the segments must cover the tile.  Returns
 * LIBRETT_SUCCESS, LIBRETT_INTERNAL_ERROR on a violation,
 * LIBRETT_INVALID_DEVICE when the candidate is not a bulk-copy tile,
 * LIBRETT_INVALID_PARAMETER for a bad problem or candidate. */
int librett_c_bulk_check(int rank, const int* dim, const int* permutation, size_t sizeofType,
                         int num_sms, int candidate);

/* librettPlan on `count` problems in order, in one call (no LibreTT
 * counterpart): for callers that create many plans, e.g. before a grouped
 * execution, without one foreign-function round trip each.  Problem k has
 * rank ranks[k], element size sizes[k], and its dims and permutation at the
 * same offset of `dims` and `perms` (the problems' arrays concatenated).
 * handles[k] receives its plan.  With synchronize nonzero every plan is
 * followed by a cudaStreamSynchronize of `stream` (as a driver that waits for
 * each plan before using it).  call_us, when not null, receives the host
 * duration of each librettPlan call (and its synchronize) in microseconds.
 * On an error the plans already made are destroyed and the error returned. */
int librett_c_plan_batch(int count, const int* ranks, const int* dims, const int* perms,
                         const size_t* sizes, void* stream, int synchronize,
                         librettHandle* handles, double* call_us);

/* The plain per-tensor loop the grouped path replaces: librettExecute on
 * each (plan, idata, odata) in order, one launch each; stops at and returns
 * the first error. */
int librett_c_execute_batch(int count, const librettHandle* plans, void* const* idata,
                            void* const* odata);
/* members, buckets (launches), members run separately, tiles, algorithmic bytes */
int librett_c_group_info(librettGroupHandle group, int* members, int* buckets, int* separate,
                         long long* tiles, long long* bytes);

/* Number of device kernel launches this library issued since load (all
 * threads, all devices).  Used to count launches inside a timed region. */
unsigned long long librett_c_launch_count(void);

/* Device memory the plan-table arena has requested since load (all
 * devices): bytes of 8 MiB slabs from cudaMalloc, table blocks handed out,
 * and bytes of large tables from its stream-ordered pool.  No LibreTT
 * counterpart (LibreTT calls cudaMalloc per plan, src/plan.cpp:1648-1676). */
int librett_c_table_arena_stats(long long* slab_bytes, long long* blocks, long long* pool_bytes);

/* Host-side fault injection, for tests of the error paths.  LibreTT exits
 * the process on a CUDA error (src/GpuUtils.h:47-56); this library returns
 * LIBRETT_INTERNAL_ERROR and stays usable.  Arms `site` so that, after
 * `after` more calls at that site succeed, the next one reports a CUDA error
 * on the host without calling the device, then disarms (after < 0 disarms
 * at once).  Sites: 0 plan-table allocation (librettPlan,
 * librettPlanMeasure), 1 a group's device image (librettGroupCreate),
 * 2 any transpose launch (librettExecute, group execution, the
 * no-allocation transpose).  Returns LIBRETT_INVALID_PARAMETER for another
 * site. */
int librett_c_inject_fault(int site, long long after);

/* Human-readable name of a result code. */
const char* librett_c_result_string(int result);

#ifdef __cplusplus
}
#endif

#endif /* LIBRETT_C_H */
