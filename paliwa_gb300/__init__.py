"""paliwa_gb300: GB300-native (sm_103a) multi-dimensional lifting-wavelet
(hierarchization) transform, a drop-in for paliwa's transform API.

The compute path is hand-written CUDA in ``csrc/`` behind the C ABI of
``include/paliwa_gb300.h``; this package is the host-side mirror of the
reference's interface (names, arguments and errors of paliwa's
paliwa_transform.hpp, paliwa_domains.hpp and paliwa_wavelets.hpp).
"""
from ._lib import (CudaError, DeviceTimeout, InvalidArgument, OutOfRange,
                   PaliwaError)
from ._lib import load as load_library
from .domains import (StridedDomain, even_strided_domain_from_domain,
                      get_strided_domains, odd_strided_domain_from_domain,
                      periodic_unit_interval_coordinates,
                      restrict_strided_with_discrete,
                      strided_domain_from_level,
                      strided_hierarchical_domain_from_level)
from .transform import (dehierarchize, dehierarchize_in, hierarchize,
                        hierarchize_in,
                        lifting_wavelet_filter_offsets_and_coefficients,
                        lifting_wavelet_reconstruct_offsets_and_coefficients,
                        transform_bounds, transform_in, transform_in_window,
                        transform_outputs,
                        wavelet_id)

__all__ = [
    "CudaError", "DeviceTimeout", "InvalidArgument", "OutOfRange",
    "PaliwaError", "load_library", "StridedDomain",
    "even_strided_domain_from_domain", "get_strided_domains",
    "odd_strided_domain_from_domain", "periodic_unit_interval_coordinates",
    "restrict_strided_with_discrete", "strided_domain_from_level",
    "strided_hierarchical_domain_from_level", "dehierarchize",
    "dehierarchize_in", "hierarchize", "hierarchize_in",
    "lifting_wavelet_filter_offsets_and_coefficients",
    "lifting_wavelet_reconstruct_offsets_and_coefficients", "transform_bounds",
    "transform_in", "transform_in_window", "transform_outputs", "wavelet_id",
]
