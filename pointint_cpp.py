"""Import name of the reference's Python module (demo/bindings.cpp: PYBIND11_MODULE(pointint_cpp)).

``import pointint_cpp`` resolves to ``pointint_gb300.pointint_cpp``.
"""
import sys

from pointint_gb300 import pointint_cpp as _impl

sys.modules[__name__] = _impl
