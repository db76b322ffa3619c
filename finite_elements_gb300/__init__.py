"""GB300 (sm_103a) assembly-and-solve path for linear triangles and tetrahedra, drop-in
for finite_elements' FiniteElementAnalysis.

The compute path is libfe_gb300.so (hand-written CUDA, C ABI in include/fe_gb300.h);
the Python modules hold the reference's object API and its list bookkeeping.
"""
from . import conditions, core, elements, loads, mesh, results  # noqa: F401
from .problem import ELASTIC, ELASTIC3D, MAGNETIC, ElementLoadSet, MagnetLoadSet, Problem  # noqa: F401

__version__ = "0.1.0"


def __getattr__(name):
    # the analysis needs the CUDA library: import it on first use so that the object
    # API and the problem generators stay importable on machines without a GPU
    if name in ("analysis", "engine"):
        import importlib
        return importlib.import_module(f".{name}", __name__)
    raise AttributeError(name)
