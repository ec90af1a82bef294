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
  /* float storage, compensated (double-float) arithmetic in registers,
   * rounded to float once per dimension; coarsest levels in FP64. */
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

#ifdef __cplusplus
}
#endif

#endif /* PALIWA_GB300_H */
