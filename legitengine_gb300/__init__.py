"""GB300-native screen-space GI path of LegitEngine (src/Render).

The product is the CUDA/C++ library built from csrc/ (lib/libgi_gb300.so) with
the C ABI of include/legit_gi.h and the C++ render-graph shim in
csrc/legit_render_graph.h.  This package only builds it and binds it.
"""
from . import build  # noqa: F401

__all__ = ["build", "gi"]
