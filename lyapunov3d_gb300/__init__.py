"""lyapunov3d_gb300 -- the lyapunov3d hot path (Lyapunov-field raymarch and
volume sweep) as hand-written CUDA for GB300 (sm_103a) behind the
reference's struct / kernel API.

* ``types``   -- ctypes mirrors of the ABI structs (structs.hpp layouts);
* ``capi``    -- the C ABI of liblyap_gb300.so (include/lyap_gb300.h);
* ``scenes``  -- seeded synthetic workloads;
* ``device``  -- device-resident frames / volumes driven through the C ABI;
* ``build``   -- compiles the library in-tree.

``capi`` (and everything that needs the library) is imported lazily so the
package can be imported to build the library.
"""
from . import types  # noqa: F401

__all__ = ["types", "scenes", "capi", "device", "build"]


def __getattr__(name):
    if name in ("capi", "device", "scenes", "build"):
        import importlib
        return importlib.import_module(f".{name}", __name__)
    raise AttributeError(name)
