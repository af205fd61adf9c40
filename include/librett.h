/*
 * librett.h -- C++ interface of the GB300 tensor-transpose engine.
 *
 * Source-compatible and link-compatible with LibreTT's public header
 * (src/librett.h:27-123 of the LibreTT project): the same type names, the
 * same enum values in the same order, and the same C++ signatures, including
 * the stream passed by reference.  Because LibreTT declares these functions
 * with C++ linkage, a caller built against LibreTT links against this
 * library's identical mangled symbols, e.g.
 *   librettPlan        -> _Z11librettPlanPjiPiS0_mRP11CUstream_st
 *   librettPlanMeasure -> _Z18librettPlanMeasurePjiPiS0_mRP11CUstream_stPvS4_
 *   librettExecute     -> _Z14librettExecutejPvS_
 *   librettDestroy     -> _Z14librettDestroyj
 *
 * Tensors are column-major (dim[0] varies fastest).  The output of a plan has
 * dimensions dim[permutation[0]], dim[permutation[1]], ... and holds
 *   out[sum_r cba[r] * idx[permutation[r]]] = in[sum_r abc[r] * idx[r]]
 * with abc[i] = prod_{j<i} dim[j] and cba[i] = prod_{j<i} dim[permutation[j]].
 * Elements are moved as raw 4-, 8- or 16-byte words, so results are bit-exact
 * copies of the input (NaN payloads included).
 *
 * Deliberate, documented divergences from LibreTT:
 *  - a CUDA error is returned as LIBRETT_INTERNAL_ERROR; LibreTT calls exit(1)
 *    (src/GpuUtils.h:47-56);
 *  - executing a plan while a different device is current returns
 *    LIBRETT_INVALID_DEVICE (LibreTT declares the code but never returns it);
 *  - rank is limited to LIBRETT_MAX_RANK (16) and the product of dims to
 *    2^40 elements; LibreTT has no explicit limit but uses 32-bit indices;
 *  - idata/odata must be aligned to min(sizeofType, 16) bytes.
 */
#ifndef LIBRETT_H
#define LIBRETT_H

#include <stddef.h>
#include <cuda_runtime.h>

#define LIBRETT_MAX_RANK 16

#ifdef __cplusplus
using librett_gpuStream_t = cudaStream_t;
#else
typedef cudaStream_t librett_gpuStream_t;
#endif

/* Handle of a plan (LibreTT src/librett.h:40). Handles increase from 0 and
 * are never reused within a process. */
typedef unsigned int librettHandle;

/* Result codes, same values as LibreTT src/librett.h:43-50. */
typedef enum librettResult_t {
  LIBRETT_SUCCESS,            /* Success */
  LIBRETT_INVALID_PLAN,       /* Invalid plan handle */
  LIBRETT_INVALID_PARAMETER,  /* Invalid input parameter */
  LIBRETT_INVALID_DEVICE,     /* Execution tried on a device other than the plan's */
  LIBRETT_INTERNAL_ERROR,     /* Internal error (includes any CUDA error) */
  LIBRETT_UNDEFINED_ERROR     /* Undefined error */
} librettResult;

#ifdef __cplusplus

/* No-op kept for source compatibility (LibreTT src/librett.h:57; there it
 * only binds an optional Umpire allocator). */
void librettInitialize();

/* No-op kept for source compatibility (LibreTT src/librett.h:62). */
void librettFinalize();

/*
 * Create a plan (LibreTT src/librett.h:78).  The plan is bound to `stream`
 * and to the device current at this call.  Planning is host-only: it fuses
 * ranks, picks a kernel and its tile, and allocates no device memory.
 */
librettResult librettPlan(librettHandle* handle, int rank, int* dim, int* permutation,
                          size_t sizeofType, librett_gpuStream_t& stream);

/*
 * Create a plan choosing among the candidates by timing each on the device
 * (LibreTT src/librett.h:96-97).  Reads idata and overwrites odata (vol *
 * sizeofType bytes each).  Synchronises `stream`.
 */
librettResult librettPlanMeasure(librettHandle* handle, int rank, int* dim, int* permutation,
                                 size_t sizeofType, librett_gpuStream_t& stream,
                                 void* idata, void* odata);

/* Destroy a plan (LibreTT src/librett.h:108). Does not synchronise. */
librettResult librettDestroy(librettHandle handle);

/*
 * Execute a plan out-of-place, asynchronously on the plan's stream
 * (LibreTT src/librett.h:121).  idata == odata -> LIBRETT_INVALID_PARAMETER.
 */
librettResult librettExecute(librettHandle handle, void* idata, void* odata);

/* ---- Grouped execution (no LibreTT counterpart) ----
 * Many plans, each with its own input and output, executed as one CUDA
 * graph: members are bucketed by kernel shape, each bucket is one launch over
 * a device-resident descriptor table.  Creation plans, allocates (stream-
 * ordered on `stream`), writes the tables and instantiates the graph
 * (synchronising `stream` once); execution is one graph launch on `stream`;
 * destruction frees in stream order.  The member plans may be destroyed once
 * the group exists (the group keeps what it needs).  Every member runs as a
 * flat tile inside its bucket (in element units when its pointers are not
 * 16-byte aligned).  Members run concurrently, so their buffers must be
 * independent: no member's output may overlap any member's input or output
 * (inputs may overlap each other).  A batch where one member reads what
 * another writes must use librettExecute in order instead; creation checks
 * the byte ranges and returns LIBRETT_INVALID_PARAMETER on an overlap. */
typedef unsigned int librettGroupHandle;

librettResult librettGroupCreate(librettGroupHandle* group, int count, const librettHandle* plans,
                                 void* const* idata, void* const* odata,
                                 librett_gpuStream_t& stream);
/* Autotunes the group's tile policy: times the policies per member size
 * class on the group's own buffers (reads idata, overwrites odata), keeps the
 * fastest and rebuilds the graph; synchronises the group's stream.  Later
 * groups over the same batch signature (members' shapes, permutations,
 * element sizes and 16-byte alignment) start from the tuned policy. */
librettResult librettGroupTune(librettGroupHandle group);
librettResult librettGroupExecute(librettGroupHandle group);
librettResult librettGroupDestroy(librettGroupHandle group);

/* One-shot: create a group on the first plan's stream, execute it once,
 * destroy it.  Prefer a persistent group when the same batch repeats. */
librettResult librettExecuteGrouped(int count, const librettHandle* plans, void* const* idata,
                                    void* const* odata);

#endif /* __cplusplus */

#endif /* LIBRETT_H */
