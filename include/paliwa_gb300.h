/*
 * paliwa_gb300: C ABI of the GB300 (sm_103a) lifting-wavelet
 * (hierarchization) transform.
 *
 * This is the boundary that the drop-in headers under include/paliwa/ (and
 * any FFI binding) call. It replaces the execution of paliwa's header-only
 * transform templates; each entry point names the reference function it
 * stands in for (file:line in the paliwa source tree).
 *
 * Conventions
 *  - Grids are dense, row-major (last dimension fastest) arrays in device
 *    memory with 2^level[d] points in dimension d, exactly the storage of a
 *    ddc::Chunk over paliwa::strided_domain_from_level(level, maximum_level)
 *    (paliwa/paliwa_domains.hpp:33-49; layout pinned by
 *    paliwa/paliwa_io.hpp:13-23 and paliwa/postprocess.py:30-35).
 *  - The caller owns every data buffer. Transforms are in place.
 *  - Every call is stream-ordered and asynchronous on `stream` (a
 *    cudaStream_t passed as void*, NULL = legacy default stream), like the
 *    reference on a Kokkos execution-space instance, which does not fence
 *    (paliwa/paliwa_transform.hpp:401-431).
 *  - No entry point throws. Each returns a status code; the message of the
 *    last failure on the calling thread is paliwa_gb_last_error(). The C++
 *    headers map the codes back to the reference's exception types.
 */
#ifndef PALIWA_GB300_H
#define PALIWA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
enum {
  PALIWA_GB_OK = 0,
  PALIWA_GB_INVALID_ARGUMENT = 1, /* std::invalid_argument / failed assert */
  PALIWA_GB_RUNTIME_ERROR = 2,    /* std::runtime_error */
  PALIWA_GB_OUT_OF_RANGE = 3,     /* std::out_of_range (unknown wavelet) */
  PALIWA_GB_CUDA_ERROR = 4,       /* a CUDA call failed */
  PALIWA_GB_TIMEOUT = 5           /* a bounded device wait gave up */
};

/* Storage and arithmetic of a grid. */
enum {
  /* double storage, double arithmetic: the reference's Value = double. */
  PALIWA_GB_F64 = 0,
  /* float storage, float arithmetic: the reference's Value = float. */
  PALIWA_GB_F32 = 1,
  /* float storage, compensated (double-float, 48-bit significand)
   * arithmetic in registers, rounded to float once per dimension. */
  PALIWA_GB_F32C = 2
};

/* Wavelets of paliwa/paliwa_wavelets.hpp:15-28. */
enum {
  PALIWA_GB_HAT = 0,
  PALIWA_GB_BIORTHOGONAL = 1,
  PALIWA_GB_FULLWEIGHTING = 2
};

/* Message of the last failed call on this thread ("" if none). */
const char *paliwa_gb_last_error(void);

/* Library ABI version (major * 10000 + minor * 100 + patch). */
int paliwa_gb_version(void);

/* Waits for the work queued on `stream` (the fence() of an execution-space
 * instance, paliwa/paliwa_utils.hpp:27-32). */
int paliwa_gb_synchronize(void *stream);

/* Wavelet name -> id. Unknown names return PALIWA_GB_OUT_OF_RANGE, as
 * lifting_wavelet_filter_offsets_and_coefficients.at(name) throws
 * std::out_of_range (paliwa/paliwa_transform.hpp:370, 397). */
int paliwa_gb_wavelet_id(const char *name, int *id);

/* Filter table of a wavelet: npasses (offset, c0, c1, c2) rows, forward
 * (direction > 0) or inverse (direction < 0), paliwa/paliwa_wavelets.hpp. */
int paliwa_gb_wavelet_filters(int wavelet, int direction, int *npasses,
                              int32_t *offsets /* [8] */,
                              double *coefficients /* [8 * 3] */);

/* Replaces paliwa::transform_in<Dim>(grid, level, maximum_level, levels,
 * filters, instance), full-grid overload, paliwa/paliwa_transform.hpp:215-251.
 * `levels` are applied in the given order, the `npasses` filters of each level
 * in table order; filter offsets other than 0 and 1 return
 * PALIWA_GB_RUNTIME_ERROR ("Filter offset not supported", :239-240). */
int paliwa_gb_transform_in(void *grid, int dtype, int ndim,
                           const int64_t *level, const int64_t *maximum_level,
                           int dim, const int64_t *levels, int nlevels,
                           const int32_t *offsets, const double *coefficients,
                           int npasses, void *stream);

/* Replaces paliwa::transform_in<Dim> (full-grid overload,
 * paliwa/paliwa_transform.hpp:215-251) on a chunk that holds only a box of
 * the level lattice, where the reference runs its bounds-checked lifting
 * passes (lifting_pass<CheckBounds = true>, :24-51, chosen at :224-228): a
 * point of a pass is updated only when it and both of its periodic
 * neighbours lie in the box; every other value is left as it is. The grid
 * holds, along dimension d, the uids window_front[d] + k * 2^(L[d] -
 * level[d]) for k < window_extents[d] (dense, row-major; the box must not
 * wrap around the period, like a DDC domain). F64 and F32 grids; levels
 * 1 <= l <= level[dim]; filter offsets other than 0 and 1 return
 * PALIWA_GB_RUNTIME_ERROR. */
int paliwa_gb_transform_in_window(void *grid, int dtype, int ndim,
                                  const int64_t *level,
                                  const int64_t *maximum_level,
                                  const int64_t *window_front,
                                  const int64_t *window_extents, int dim,
                                  const int64_t *levels, int nlevels,
                                  const int32_t *offsets,
                                  const double *coefficients, int npasses,
                                  void *stream);

/* Replaces paliwa::hierarchize_in<Dim> / dehierarchize_in<Dim>
 * (paliwa/paliwa_transform.hpp:346-399): levels level[dim] .. lmin+1
 * (forward) or lmin+1 .. level[dim] (inverse) with the wavelet's table.
 * Requires 0 <= minimum_level <= level <= maximum_level (:359-362). */
int paliwa_gb_hierarchize_in(void *grid, int dtype, int ndim,
                             const int64_t *level,
                             const int64_t *minimum_level,
                             const int64_t *maximum_level, int dim,
                             int wavelet, void *stream);
int paliwa_gb_dehierarchize_in(void *grid, int dtype, int ndim,
                               const int64_t *level,
                               const int64_t *minimum_level,
                               const int64_t *maximum_level, int dim,
                               int wavelet, void *stream);

/* Replaces paliwa::hierarchize / dehierarchize
 * (paliwa/paliwa_transform.hpp:401-431): every dimension in order, 0 first. */
int paliwa_gb_hierarchize(void *grid, int dtype, int ndim,
                          const int64_t *level, const int64_t *minimum_level,
                          const int64_t *maximum_level, int wavelet,
                          void *stream);
int paliwa_gb_dehierarchize(void *grid, int dtype, int ndim,
                            const int64_t *level,
                            const int64_t *minimum_level,
                            const int64_t *maximum_level, int wavelet,
                            void *stream);

/* ------------------------------------------------------------------------
 * Restricted-output transform along one axis.
 *
 * Replaces paliwa::transform_bounds (paliwa/paliwa_domains.hpp:357-452):
 * the exact access sets of the lifting sequence `levels` x passes (only the
 * filter offsets matter) that make the output interval
 * [outputs_min, outputs_max] (finest-level uids, min > max wraps, min < 0
 * empty) exact. bounds receives 2 * (level + 1) values: the required input
 * bounds (min, max) per hierarchical level 0..level, -1 -1 where empty.
 * writes (optional, may be NULL) receives 2 * nlevels * nfilters values: the
 * write bounds of each (level index, pass). Host-only: touches no GPU. */
int paliwa_gb_transform_bounds(int64_t outputs_min, int64_t outputs_max,
                               int64_t level, int64_t maximum_level,
                               const int64_t *levels, int nlevels,
                               const int32_t *offsets, int nfilters,
                               int64_t *bounds, int64_t *writes);

/* Replaces paliwa::transform_in(grid, level, maximum_level, levels, filters,
 * outputs, exec, PoleExecution) (paliwa/paliwa_transform.hpp:333-344, via
 * detail::transform_with_remote :258-331): the lifting sequence along `dim`
 * restricted to the points that the outputs depend on. Leaves the buffer as
 * the reference leaves its grid: outputs exact, the dependency cone holding
 * the intermediate values, everything else untouched.
 * The grid is a window buffer (F64 or F32): along dimension d it holds the
 * uids (window_front[d] + k * 2^(L[d] - level[d])) mod 2^L[d] for
 * k < window_extents[d], dense and row-major; the full grid is front 0,
 * extents 2^level. Windows may wrap around the period, so one buffer can hold
 * a slab and its periodic halo. outputs_* describe a strided domain in uids
 * (front in [0, 2^L), extents, strides); along `dim` it sets the output
 * interval, in the other dimensions the transformed columns, which must be
 * grid points inside the window. Errors: PALIWA_GB_INVALID_ARGUMENT for
 * shapes and levels (std::invalid_argument), PALIWA_GB_RUNTIME_ERROR when a
 * required input lies outside the window ("Transform domain is missing
 * required input values", :282-289). Empty outputs return at once. */
int paliwa_gb_transform_outputs(
    void *grid, int dtype, int ndim, const int64_t *level,
    const int64_t *maximum_level, const int64_t *window_front,
    const int64_t *window_extents, int dim, const int64_t *levels,
    int nlevels, const int32_t *offsets, const double *coefficients,
    int nfilters, const int64_t *outputs_front,
    const int64_t *outputs_extents, const int64_t *outputs_strides,
    void *stream);

/* Replaces paliwa::dump_chunk_span_to_binary_file (paliwa/paliwa_io.hpp:13-23):
 * writes `bytes` bytes of device memory at `data` (a grid's dense row-major
 * storage) to `filename`, truncating it, in storage order with no header --
 * the raw format paliwa/postprocess.py reads with numpy.fromfile. The copy is
 * ordered after the work already queued on `stream`; the call returns once
 * the file is written. PALIWA_GB_RUNTIME_ERROR if the file cannot be opened
 * or written. */
int paliwa_gb_dump_to_binary_file(const void *data, int64_t bytes,
                                  const char *filename, void *stream);

/* The transform of paliwa_gb_hierarchize (direction 1) or
 * paliwa_gb_dehierarchize (direction -1) without any device allocation.
 * No counterpart in the reference: it is for callers that cannot let a
 * library allocate device memory -- programs whose own allocator already
 * holds the GPU's memory (a framework's caching pool, a solver's arena),
 * where a library allocation can fail or fragment it, and time-step loops
 * that cannot pay for allocator calls or cudaFree's device synchronization.
 * Only grids with a pencil longer than 4096 points need scratch; this entry
 * point takes it from one 64 MiB array in device memory that every GPU
 * loading the library holds until the process exits, so such grids may be at
 * most 64 MiB (larger ones return PALIWA_GB_INVALID_ARGUMENT before any work
 * is queued). The first call on each device looks up that array's address
 * (cudaGetSymbolAddress) with the device current; make it before any stream
 * capture. All calls share the array, which keeps the last call's contents
 * (the transform writes every byte it reads back, so nothing is cleared):
 * calls whose work overlaps on the GPU (different streams) race on it and
 * must be ordered by the caller. */
int paliwa_gb_transform_noalloc(void *grid, int dtype, int ndim,
                                const int64_t *level,
                                const int64_t *minimum_level,
                                const int64_t *maximum_level, int wavelet,
                                int direction, void *stream);

/* ------------------------------------------------------------------------
 * Batched transforms of many component grids.
 *
 * Replaces the per-grid loop of the reference's combination-technique driver,
 * paliwa::hierarchize(grid_i, level_i, lmin, lmax, wavelet, instances[i % n])
 * (test/test_paliwa_combination_technique.cpp:164-174), and its
 * dehierarchize counterpart. grid_ptrs[i] is the device address of grid i
 * (dense row-major, 2^sum(levels[i*ndim .. i*ndim+ndim-1]) values of dtype);
 * the pointers are bound at creation. Each direction's launches are captured
 * into a CUDA graph on first use on a non-default stream and replayed.
 */
typedef struct paliwa_gb_batch paliwa_gb_batch;

int paliwa_gb_batch_create(int ndim, int ngrids, const int64_t *levels,
                           const int64_t *minimum_level,
                           const int64_t *maximum_level, int dtype,
                           int wavelet, void *const *grid_ptrs,
                           paliwa_gb_batch **out);
int paliwa_gb_batch_hierarchize(paliwa_gb_batch *batch, void *stream);
int paliwa_gb_batch_dehierarchize(paliwa_gb_batch *batch, void *stream);
/* enable != 0 (default): capture and replay CUDA graphs. */
int paliwa_gb_batch_use_graphs(paliwa_gb_batch *batch, int enable);
/* Splits the batch into `ngroups` groups of about equal size (grids dealt
 * largest first), each planned on its own and run on its own branch (forked
 * streams, joined into the caller's stream), so that the groups' launches
 * overlap; creation uses 4 (fewer when there are fewer grids). 1 runs every
 * launch on the caller's stream. Re-plans both directions (the autotuner's
 * choices are kept) after synchronizing the device. No counterpart in the
 * reference (its CT driver spreads grids over execution-space instances,
 * test/test_paliwa_combination_technique.cpp:164-174). */
int paliwa_gb_batch_set_groups(paliwa_gb_batch *batch, int ngroups);
/* enable != 0 (default): grids whose trailing axes span blocks ("slabs") of
 * at most 32 KB, with levels to transform along two or more of those axes,
 * transform all of them in one launch of the slab kernel (one HBM pass over
 * the grid, tiles moved by the tensor memory accelerator); 0 plans every
 * axis on its own. Results are the same bits either way. Re-plans both
 * directions after synchronizing the device. No counterpart in the
 * reference. */
int paliwa_gb_batch_use_slabs(paliwa_gb_batch *batch, int enable);
/* enable != 0 (default): FP32-compensated stages of strided pencils of up
 * to 2048 points (up to 128 chunks; inner extent of 4 or more columns, or
 * of 2 with the pencil pairs one after another) and of the last axis'
 * pencils of up to 4096 points, in 16-byte aligned grids,
 * may run on the TMA wide kernel: the wide kernel's register transform,
 * with each tile moved between HBM and shared memory by bulk tensor copies
 * over a tensor map of the grid's axis (bounded waits, reported by
 * paliwa_gb_batch_status). It is the planner's default for them except the
 * strided 4-point chunks, which stay an autotuner choice. 0 keeps every
 * such stage on the wide, tile or staged kernel's per-thread copies.
 * Results are the same bits either way. Re-plans both directions after
 * synchronizing the device. No counterpart in the reference. */
int paliwa_gb_batch_use_tma(paliwa_gb_batch *batch, int enable);
/* ctas > 0 caps every launch of the batch at that many CTAs per SM (the
 * kernels are persistent: by default a launch takes every slot that fits),
 * which leaves room on each SM for the launches of the batch's other
 * groups; 0 (default) restores the default. Re-plans both directions after
 * synchronizing the device. No counterpart in the reference. */
int paliwa_gb_batch_set_ctas_per_sm(paliwa_gb_batch *batch, int ctas);
/* PALIWA_GB_TIMEOUT if a slab launch of this batch gave up a bounded wait
 * for its tile copies since the last call (the flag is then cleared);
 * otherwise PALIWA_GB_OK. Synchronizes with the device. */
int paliwa_gb_batch_status(paliwa_gb_batch *batch);
int paliwa_gb_batch_info(const paliwa_gb_batch *batch, int64_t *points,
                         int64_t *launches_forward,
                         int64_t *launches_inverse);
/* Runs one direction (forward != 0: hierarchize) launch by launch with CUDA
 * events around each launch, waits for it, and reports each launch's
 * duration, algorithmic bytes (one read and one write of every grid point
 * it stores) and kernel: R > 0 the staged kernel with chunks of R points,
 * -R the direct kernel (pencils in registers), 64 + R and 128 + R the wide
 * kernel (rows of adjacent columns in registers) on a strided axis and on
 * the last axis, 192 + R and 256 + R the tile kernel (row-major tiles in
 * shared memory, rows of adjacent columns in registers) for pencils of up to
 * 32 chunks and longer ones, 512 the halo pass before a windowed stage
 * (its bytes count one read and one write of each point it copies), 1024
 * the slab kernel (every level of a grid's
 * trailing axes in one pass; its bytes count one read and one write of each
 * point), 2048 + R the TMA wide kernel (+ 32: pencils of 8 to 32 chunks,
 * + 64: more, + 96: the last axis, + 160: its pencils of more than 32
 * chunks, + 128: inner extent 2); `kernels` may be null. Call with
 * capacity 0 to get *nlaunches first. */
int paliwa_gb_batch_profile(paliwa_gb_batch *batch, int forward, void *stream,
                            int capacity, int *nlaunches, float *ms,
                            int64_t *bytes, int32_t *kernels);
/* Autotuner: for each direction, first slab launches against the same
 * axes planned one by one (when paliwa_gb_batch_use_slabs allows slabs;
 * either way round, the faster kept), then each class of periodic stages
 * (last axis or strided, sub-lattice or not, pencil length, inner extent)
 * and each kernel that applies to it (staged, direct, wide, tile),
 * re-plans and times the whole direction (best of `reps` event-timed runs,
 * executed as the batch executes it: its groups on parallel branches, from
 * a graph when graphs are on) and keeps the fastest choice; classes are tried one after another (coordinate
 * descent from the planner's defaults; classes holding under 2 % of the
 * points are left at the default). Runs the transforms on the batch's
 * grids: every timed direction is paired with its inverse, so the contents
 * come back up to rounding (bit-exact for FP64 and FP32 only if the
 * transform pair is exact on them). Synchronises with the stream. *changed
 * (may be null) = classes whose kernel changed, plus directions whose slab
 * choice changed. Takes a second or more for
 * a large batch; graphs are re-captured on the next run. No counterpart in
 * the reference, which has no kernel choice to make. */
int paliwa_gb_batch_autotune(paliwa_gb_batch *batch, void *stream, int reps,
                             int *changed);
/* The classes of periodic stages of one direction's plan: class code
 * (bit 0 last axis, bit 1 sub-lattice of a long pencil, bits 2-7 log2 of the
 * pencil length, bits 8-11 log2 of the inner extent in bytes, capped at 8),
 * the kernels that apply (bit c for c = 0 staged with 16-point chunks,
 * 1 direct, 2 wide, 3 tile, 4 staged with 32-point chunks, 5 the TMA wide
 * kernel) and the chosen
 * one. Call with capacity 0 to get *nclasses first. */
int paliwa_gb_batch_tuning(const paliwa_gb_batch *batch, int forward,
                           int capacity, int *nclasses, int32_t *classes,
                           int32_t *kernels, int32_t *choices);
/* Sets the kernel of `nclasses` classes of one direction's plan (codes and
 * kernel numbers as paliwa_gb_batch_tuning reports them) and re-plans that
 * direction, e.g. to replay an earlier autotuner result without timing.
 * PALIWA_GB_INVALID_ARGUMENT, with nothing changed, when a class has no
 * stage in the batch or the kernel does not apply to it. Every kernel gives
 * the same results. */
int paliwa_gb_batch_set_tuning(paliwa_gb_batch *batch, int forward,
                               int nclasses, const int32_t *classes,
                               const int32_t *choices);
void paliwa_gb_batch_destroy(paliwa_gb_batch *batch);

/* ------------------------------------------------------------------------
 * Combination technique: sparse-grid combine, restrict and full-grid scatter
 * in FP64. Restates test/test_paliwa_combination_technique.cpp:176-318
 * (there only a test driver): every hierarchical subspace 0 <= s <= l of
 * every grid is counted (paliwa/paliwa_utils.hpp:9-26); subspaces present in
 * more than one grid are kept (keep_all != 0 keeps all), ordered
 * lexicographically, each stored densely over the extents of
 * paliwa::strided_hierarchical_domain_from_level(s, maximum_level)
 * (paliwa/paliwa_domains.hpp:51-83), concatenated.
 */
typedef struct paliwa_gb_ct paliwa_gb_ct;

int paliwa_gb_ct_create(int ndim, int ngrids, const int64_t *levels,
                        const double *coefficients,
                        const int64_t *maximum_level, int dtype,
                        void *const *grid_ptrs, int keep_all,
                        paliwa_gb_ct **out);
int paliwa_gb_ct_info(const paliwa_gb_ct *ct, int64_t *npoints,
                      int64_t *nsubspaces);
/* levels: nsubspaces * ndim; offsets: nsubspaces (first point of each). */
int paliwa_gb_ct_subspaces(const paliwa_gb_ct *ct, int64_t *levels,
                           int64_t *offsets);
/* sparse[p] = sum over grids g containing the subspace, in grid order, of
 * coefficient_g * grid_g[p] (:256-290). sparse is device memory of npoints
 * doubles; it is overwritten. */
int paliwa_gb_ct_combine(paliwa_gb_ct *ct, double *sparse, void *stream);
/* Writes each kept subspace's combined value into every grid containing it
 * (rounded to the grid's storage type). */
int paliwa_gb_ct_restrict(paliwa_gb_ct *ct, const double *sparse,
                          void *stream);
/* full = 0, then full[subspace points] += sparse (:293-318); full is the
 * dense grid at maximum_level (2^sum(maximum_level) doubles). */
int paliwa_gb_ct_scatter(paliwa_gb_ct *ct, const double *sparse, double *full,
                         void *stream);
void paliwa_gb_ct_destroy(paliwa_gb_ct *ct);

#ifdef __cplusplus
}
#endif

#endif /* PALIWA_GB300_H */
