"""CPU oracle for the focal-stencil path -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.

The oracle is a float64 numpy/scipy restatement of vibespatial-raster's own
CPU algorithms (and, where the reference only has a GPU kernel, of that
kernel's arithmetic).  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline legs of ``bench.py`` may import it, and only as the checker or
the timed CPU baseline.  The product path (``vsr_gb300``) never imports it.

Parity is pinned: ``tests/test_oracle_golden.py`` checks every function
here against golden vectors produced by the reference's own CPU code
(``tests/golden/make_golden.py``).  The normalised convolution has no CPU
path in the reference, so it is pinned against a literal loop restatement of
the reference kernel plus the reference's known-answer tests.
"""

from oracle.focal_oracle import (  # noqa: F401
    CURVATURE,
    FOCAL_STATS,
    TPI,
    TRI,
    cellsize_from_affine,
    convolve_normalized,
    convolve_normalized_loop,
    focal_mean,
    focal_stat,
    gaussian_weights,
    hillshade,
    nodata_mask,
    nodata_ring,
    slope_aspect,
    slope_aspect_center_only,
    terrain_derivative,
    terrain_out_dtype,
)
