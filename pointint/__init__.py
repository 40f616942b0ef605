"""Import name of the reference's Python package (pointint).

Only ``pointint.core`` is provided: the Fourier intersection-volume path as a
torch layer over the GB300 library (``pointint_gb300``).  The reference's
simulator, viewer and scripts are not part of this path.
"""
