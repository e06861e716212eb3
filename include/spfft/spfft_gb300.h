/* Extensions of this GB300 library beyond the reference's C interface. None of these functions has
 * a counterpart in the reference; each says what it adds. All return SpfftError. */
#ifndef SPFFT_GB300_H
#define SPFFT_GB300_H

#include "spfft/config.h"
#include "spfft/errors.h"
#include "spfft/transform.h"
#include "spfft/transform_float.h"
#include "spfft/types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Host-only index planning: the z-stick layout a transform of these parameters uses. Runs without
 * a GPU. valueIndices receives numLocalElements ints (stick * dimZ + z per value, in input order),
 * stickKeys receives up to maxSticks ints (sorted x * dimY + y storage keys); numSticks and
 * zeroZeroStick (position of key 0, or numSticks if absent) may be NULL. Errors are those of
 * transform creation (invalid indices, invalid parameters). */
SPFFT_EXPORT SpfftError spfft_gb300_plan_indices(SpfftTransformType transformType, int dimX,
                                                 int dimY, int dimZ, int numLocalElements,
                                                 const int* indices, int* valueIndices,
                                                 int* stickKeys, int maxSticks, int* numSticks,
                                                 int* zeroZeroStick);

/* Every table of the index plan a transform of these parameters uses, for verification: from the
 * host planner (planner 0) or from the device planner on the current device (planner 1; where it
 * declines -- duplicate triplets, very large key or position ranges -- the host planner runs and
 * *usedDevice is 0). `tables` receives, back to back: numSticks, numColumns, zeroZeroStick,
 * identityOrder, valueIndices[numLocalElements], stickKeys[numSticks], stickColumn[numSticks],
 * stickY[numSticks], stickPlanePos[numSticks], columnX[numColumns],
 * columnStickStart[numColumns + 1], entryPos[numLocalElements], entryUser[numLocalElements],
 * stickEntryStart[numSticks + 1] and, for R2C, hermitianWeight[numLocalElements]. *size receives
 * the number of ints; nothing is written to `tables` when it is NULL or `capacity` is smaller.
 * Errors are those of transform creation. */
SPFFT_EXPORT SpfftError spfft_gb300_plan_tables(int planner, SpfftTransformType transformType,
                                                int dimX, int dimY, int dimZ,
                                                int numLocalElements, const int* indices,
                                                int* tables, long long capacity, long long* size,
                                                int* usedDevice);

/* Fault injection for tests of the allocation-failure paths (no GPU fault involved): the next
 * afterAllocations device or pinned host allocations of the library succeed and the one after fails
 * once, as if the CUDA allocator had failed (SPFFT_GPU_ALLOCATION_ERROR for device memory,
 * SPFFT_ALLOCATION_ERROR for pinned host memory). -1 turns it off. previous (may be NULL) receives
 * the countdown before the call: -1 once an injected failure has fired. */
SPFFT_EXPORT SpfftError spfft_gb300_inject_allocation_failure(int afterAllocations, int* previous);

/* Number of live index plans that transform creation can share (transforms created with the same
 * type, sizes and index triplets on the same device share one plan and its device tables;
 * SPFFT_GB300_PLAN_CACHE=0 turns the sharing off). */
SPFFT_EXPORT SpfftError spfft_gb300_plan_cache_size(int* count);

/* Attach a CUDA stream (a cudaStream_t passed as void*). Afterwards every call of the transform is
 * enqueued on that stream only: no internal stream and no ordering against the legacy default
 * stream. In SPFFT_EXEC_ASYNCHRONOUS mode calls then return without waiting, which makes them
 * usable inside CUDA graph capture. NULL restores the default protocol. */
SPFFT_EXPORT SpfftError spfft_gb300_transform_set_stream(SpfftTransform transform, void* stream);
SPFFT_EXPORT SpfftError spfft_gb300_float_transform_set_stream(SpfftFloatTransform transform,
                                                               void* stream);

/* Kernel-only execution on device pointers and a given stream: no pointer inspection, no copies,
 * no synchronisation, no preceding-error check. values: interleaved complex frequency values;
 * space: the space domain in the layout of the transform. */
SPFFT_EXPORT SpfftError spfft_gb300_transform_backward_device(SpfftTransform transform,
                                                              const double* values, double* space,
                                                              void* stream);
SPFFT_EXPORT SpfftError spfft_gb300_transform_forward_device(SpfftTransform transform,
                                                             const double* space, double* values,
                                                             SpfftScalingType scaling,
                                                             void* stream);
SPFFT_EXPORT SpfftError spfft_gb300_float_transform_backward_device(SpfftFloatTransform transform,
                                                                    const float* values,
                                                                    float* space, void* stream);
SPFFT_EXPORT SpfftError spfft_gb300_float_transform_forward_device(SpfftFloatTransform transform,
                                                                   const float* space,
                                                                   float* values,
                                                                   SpfftScalingType scaling,
                                                                   void* stream);

/* Adjoints for differentiation (no counterpart in the reference), on device pointers and `stream`,
 * without synchronisation. Gradients follow the convention dL/dRe + i dL/dIm for complex
 * quantities. adjoint_backward maps the gradient of the space domain to the gradient of the
 * frequency values: for C2C the unnormalised forward transform and its gather (the transpose of
 * the backward scatter); for R2C the same times each value's hermitian multiplicity (2, or 1 for
 * self-conjugate frequencies, the x Nyquist plane and the y Nyquist row of the x = 0 plane).
 * adjoint_forward maps the gradient of the frequency values to the gradient of the space domain
 * (the backward transform of the value gradient divided by those multiplicities, scaled like the
 * forward). The R2C adjoints assume each hermitian pair is given once, as the reference's R2C
 * index rules describe. */
SPFFT_EXPORT SpfftError spfft_gb300_transform_adjoint_backward(SpfftTransform transform,
                                                               const double* gradSpace,
                                                               double* gradValues, void* stream);
SPFFT_EXPORT SpfftError spfft_gb300_transform_adjoint_forward(SpfftTransform transform,
                                                              const double* gradValues,
                                                              double* gradSpace,
                                                              SpfftScalingType scaling, void* stream);
SPFFT_EXPORT SpfftError spfft_gb300_float_transform_adjoint_backward(SpfftFloatTransform transform,
                                                                     const float* gradSpace,
                                                                     float* gradValues, void* stream);
SPFFT_EXPORT SpfftError spfft_gb300_float_transform_adjoint_forward(SpfftFloatTransform transform,
                                                                    const float* gradValues,
                                                                    float* gradSpace,
                                                                    SpfftScalingType scaling,
                                                                    void* stream);

/* Profiling aid: run one backward (direction 0: input = values, output = space) or forward
 * (direction 1: input = space, output = values) on device pointers and `stream`, with CUDA events
 * around each of the three kernels of the pass; waits and writes the three kernel times (ms) to
 * stageMs. The pass order is z, y, x for backward and x, y, z for forward. */
SPFFT_EXPORT SpfftError spfft_gb300_transform_stage_times(SpfftTransform transform, int direction,
                                                          const double* input, double* output,
                                                          SpfftScalingType scaling, void* stream,
                                                          float* stageMs);
SPFFT_EXPORT SpfftError spfft_gb300_float_transform_stage_times(SpfftFloatTransform transform,
                                                                int direction, const float* input,
                                                                float* output,
                                                                SpfftScalingType scaling,
                                                                void* stream, float* stageMs);

/* Which kernels a transform runs (no counterpart in the reference): bit 0 set = size-specialised
 * z pass; bit 1 set = fused size-specialised plane pass (y and x in one kernel per plane); bit 2
 * set = split size-specialised y and x passes over column and row groups; otherwise the generic
 * kernels. The plane strategy can be forced at transform creation with the environment variable
 * SPFFT_GB300_PLANE=fused|split|generic. */
SPFFT_EXPORT SpfftError spfft_gb300_transform_path_info(SpfftTransform transform, int* flags);
SPFFT_EXPORT SpfftError spfft_gb300_float_transform_path_info(SpfftFloatTransform transform,
                                                              int* flags);

/* Autotuner (no counterpart in the reference). Times `repetitions` backward + scaled forward pairs
 * of every valid tile shape and plane strategy of the transform (first the sticks per z block with
 * the current plane strategy, then the fused plane pass with each chunk size and thread count and
 * the split passes with each column / row group size, then the split of each specialised z and
 * split-y pass, spfft_gb300_transform_split_stages, then the radix plans of the lengths that run
 * on the generic kernels, spfft_gb300_transform_radix_plans) on the transform's own device buffers,
 * and keeps the fastest; writes its time per pair in milliseconds to msPerPair (may be NULL).
 * Synchronous; overwrites the grid's internal device space-domain buffer; no other call on the
 * transform may run meanwhile. The choice lasts for the transform (clones start from the default
 * choice). */
SPFFT_EXPORT SpfftError spfft_gb300_transform_autotune(SpfftTransform transform, int repetitions,
                                                       float* msPerPair);
SPFFT_EXPORT SpfftError spfft_gb300_float_transform_autotune(SpfftFloatTransform transform,
                                                             int repetitions, float* msPerPair);
/* The tile shapes the transform runs with: tuning[0] sticks per z block (0: generic z kernels),
 * [1] plane strategy (0 generic, 1 fused, 2 split), [2] fused: half the x chunk rows, [3] fused:
 * threads per block, [4] split: columns per y block, [5] split: rows per x block. */
SPFFT_EXPORT SpfftError spfft_gb300_transform_tuning(SpfftTransform transform, int* tuning);
SPFFT_EXPORT SpfftError spfft_gb300_float_transform_tuning(SpfftFloatTransform transform, int* tuning);
/* Split plane passes: rows per block of the x backward kernel, which the autotuner chooses apart
 * from the x forward kernel's (tuning[5]; it holds the compact rows besides the FFT rows, so fewer
 * rows can let more blocks share an SM); 0 when the plane passes are not split. Starts equal to
 * tuning[5] (SPFFT_GB300_XB_ROWS=n at transform creation sets n, where n is a candidate). */
SPFFT_EXPORT SpfftError spfft_gb300_transform_x_backward_rows(SpfftTransform transform, int* rows);
SPFFT_EXPORT SpfftError spfft_gb300_float_transform_x_backward_rows(SpfftFloatTransform transform, int* rows);

/* The radix plans of the z, y and x lengths: numStages[d] stages with radices
 * radices[d * 24 + 0 .. numStages[d] - 1] (d = 0 z, 1 y, 2 x; 24 slots per length). For a length
 * on the generic (runtime-radix) kernels, the autotuner chooses among several plans (the default
 * grouping of powers of two into radix 8, the reverse order, radix-4 and radix-2 stages). For a
 * length on the size-specialised kernels, the radices of the two- or three-pass split its backward
 * pass runs (of the complex FFT length: half the x length for the x pass of an R2C transform);
 * spfft_gb300_transform_split_stages gives every pass. */
/* Splits of the size-specialised kernels (no counterpart in the reference): radices[0..5]
 * = the first-pass radix A of the split A x B (A * B = the pass's complex FFT length) that the z
 * backward, z forward, y backward, y forward, x backward and x forward passes run, 0 for a pass on
 * the generic kernels. The z passes and the split y passes are built in both orders of their two
 * radices wherever the orders differ (192: 12 x 16 and 16 x 12), and, in double precision for the
 * lengths whose second radix is 12 or 16 (144, 180, 192, 256), as a three-pass split A x B1 x B2
 * that runs the B-point DFTs as two shared-memory passes (192: 12 x 4 x 4); the autotuner chooses
 * one per pass, and SPFFT_GB300_SPLITS=zb,zf,yb,yf (each 0 for the default order, 1 for the swapped
 * one, 2 for the three-pass split) at transform creation sets them. The fused plane kernels and
 * the x passes have one fixed split. */
SPFFT_EXPORT SpfftError spfft_gb300_transform_splits(SpfftTransform transform, int* radices);
SPFFT_EXPORT SpfftError spfft_gb300_float_transform_splits(SpfftFloatTransform transform, int* radices);
/* Every radix of those splits (no counterpart in the reference): stages[3 * pass + 0..2] for the
 * six passes in the order above, (A, B, 0) for a two-pass split, (A, B1, B2) for a three-pass split,
 * (0, 0, 0) for a pass on the generic kernels. */
SPFFT_EXPORT SpfftError spfft_gb300_transform_split_stages(SpfftTransform transform, int* stages);
SPFFT_EXPORT SpfftError spfft_gb300_float_transform_split_stages(SpfftFloatTransform transform, int* stages);
SPFFT_EXPORT SpfftError spfft_gb300_transform_radix_plans(SpfftTransform transform, int* numStages,
                                                          int* radices);
SPFFT_EXPORT SpfftError spfft_gb300_float_transform_radix_plans(SpfftFloatTransform transform,
                                                                int* numStages, int* radices);

/* ---- batched execution (no counterpart in the reference; the GB300 form of its multi-transform)
 * A batch holds many transforms (all double or all float, on distinct grids, same device). Each
 * pass of each group of equally shaped transforms runs as ONE kernel launch over all of them, so
 * small transforms fill the GPU; different groups run concurrently on forked streams. Buffers are
 * bound once; a backward + forward pair can be captured into a CUDA graph on first use and
 * replayed. Transforms whose lengths have no specialised kernels run one by one inside the same
 * calls. */
typedef void* SpfftGb300Batch;
SPFFT_EXPORT SpfftError spfft_gb300_batch_create(SpfftGb300Batch* batch, int numTransforms,
                                                 const SpfftTransform* transforms);
SPFFT_EXPORT SpfftError spfft_gb300_float_batch_create(SpfftGb300Batch* batch, int numTransforms,
                                                       const SpfftFloatTransform* transforms);
SPFFT_EXPORT SpfftError spfft_gb300_batch_destroy(SpfftGb300Batch batch);
/* values[i]: device interleaved-complex frequency values of transform i; spaces[i]: its device
 * space domain. Pointers must be aligned to the complex size (16 bytes double, 8 bytes float).
 * Synchronous: call it while no work of the batch is in flight. Captured graphs stay valid, except
 * when the buffers of a transform that runs unbatched change: those graphs are captured anew. */
SPFFT_EXPORT SpfftError spfft_gb300_batch_bind(SpfftGb300Batch batch, void* const* values,
                                               void* const* spaces);
SPFFT_EXPORT SpfftError spfft_gb300_batch_backward(SpfftGb300Batch batch, void* stream);
SPFFT_EXPORT SpfftError spfft_gb300_batch_forward(SpfftGb300Batch batch, SpfftScalingType scaling,
                                                  void* stream);
/* Backward then forward of every transform as one CUDA graph on `stream` (not the default
 * stream). The graph is captured on the first call for each scaling and replayed afterwards; it
 * reads the bound pointers from a device table, so it follows later rebinds. */
SPFFT_EXPORT SpfftError spfft_gb300_batch_pair_graph(SpfftGb300Batch batch, SpfftScalingType scaling,
                                                     void* stream);
SPFFT_EXPORT SpfftError spfft_gb300_batch_info(SpfftGb300Batch batch, int* numGroups,
                                               int* numUnbatched, int* launchesPerPair);
/* Autotuner of a bound batch: for each group of equally shaped transforms, times `repetitions`
 * backward + scaled forward pairs of the group alone on `stream` for each plane strategy that fits
 * (fused, split) and each sticks-per-z-block size, then for each row-group count of a fused group
 * (spfft_gb300_batch_row_groups), and keeps the fastest. Overwrites the contents of
 * the bound buffers; drops captured graphs (the next graph call captures anew). Writes the sum of
 * the groups' best times per pair in milliseconds to msPerPair (may be NULL). Synchronous. */
SPFFT_EXPORT SpfftError spfft_gb300_batch_autotune(SpfftGb300Batch batch, int repetitions, void* stream,
                                                   float* msPerPair);
/* How transform `index` (its position at creation) runs: 0 one by one (no batched kernels for its
 * lengths), 1 batched with split y and x passes, 2 batched with one fused plane pass (y and x per
 * plane with the compact plane on chip; chosen for cubic planes that fit two blocks per SM, or
 * forced with SPFFT_GB300_BATCH_PLANE=fused|split at batch creation). */
SPFFT_EXPORT SpfftError spfft_gb300_batch_transform_path(SpfftGb300Batch batch, int index, int* path);
/* Row groups of the fused plane passes of transform `index`: the x pass of each plane block is
 * split into this many independent groups of warps that synchronise only among themselves (0 when
 * the transform's plane passes are not fused). Chosen by spfft_gb300_batch_autotune, or set at
 * batch creation with SPFFT_GB300_BATCH_ROW_GROUPS=1|2|3|4 where valid; by default 4 in FP32
 * (where valid) and 1 in FP64. */
SPFFT_EXPORT SpfftError spfft_gb300_batch_row_groups(SpfftGb300Batch batch, int index, int* groups);
/* One direction (0 backward, 1 forward) of the bound batch with the groups run pass by pass on
 * `stream` and events between the three passes (z, y, x in backward order; a fused group runs its
 * plane pass in the y slot and nothing in the x slot); waits and writes the pass times in
 * milliseconds to stageMs[3]. For profiling: ordinary calls run groups concurrently. */
SPFFT_EXPORT SpfftError spfft_gb300_batch_stage_times(SpfftGb300Batch batch, int direction,
                                                      SpfftScalingType scaling, void* stream,
                                                      float* stageMs);

/* Multi-transform calls (spfft_multi_transform_* and spfft_float_multi_transform_*) run as one
 * batched execution (the batch above, built and cached by the library, its graphs replayed) when
 * the call has at least two transforms, all on one device, none with a stream set by
 * spfft_gb300_*transform_set_stream, every buffer device memory or pinned host memory, complex-
 * aligned, and one scaling for all forwards. Otherwise the transforms run one by one. This counts
 * the calls so far that ran batched (process-wide). */
SPFFT_EXPORT SpfftError spfft_gb300_multi_batched_calls(long long* count);

/* Allocation-free backward transform (no counterpart in the reference). Runs the backward transform
 * of an existing double-precision transform on device pointers (values: interleaved complex
 * frequency values; space: the space domain in the transform's layout) on `stream` (a
 * cudaStream_t; NULL is the default stream), keeping the z-stick and plane intermediates in a
 * static 64 MiB device array that is part of the library, instead of memory the library allocates.
 * For callers that cannot let the library call cudaMalloc: applications whose device memory is
 * owned and budgeted by their own pool or arena allocator, latency-critical loops that cannot
 * afford an allocation's device synchronisation, plug-ins whose host application forbids them to
 * allocate. The call allocates nothing and does not synchronise.
 * Limits and rules:
 *  - values and space must be device memory of the transform's GPU (there is no staging through
 *    host memory); anything else is rejected with SPFFT_INVALID_PARAMETER_ERROR before any launch;
 *  - a CUDA error pending from earlier work is reported as SPFFT_GPU_PRECEDING_ERROR;
 *  - transforms whose intermediates exceed 64 MiB are rejected with SPFFT_INVALID_PARAMETER_ERROR;
 *  - every GPU that loads the library holds the 64 MiB array until the process exits;
 *  - all calls share the one array per GPU: calls that overlap on the GPU (different streams, or
 *    different transforms in flight at once) race and corrupt each other's results;
 *  - the first call on each device (and the first after the device's context was reset) looks up
 *    the array's device address; make that first call before any stream capture. */
SPFFT_EXPORT SpfftError spfft_gb300_transform_backward_noalloc(SpfftTransform transform,
                                                               const double* values,
                                                               double* space, void* stream);

#ifdef __cplusplus
}
#endif
#endif
