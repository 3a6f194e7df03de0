"""GB300-native (sm_103a) acoustic ray-tracing core, a drop-in for the
ray-tracing path of E.A.R (Evaluation of Acoustics using Ray-tracing).

The compute path is the C-ABI library ``lib/libear_gb300.so`` (LBVH build,
stackless traversal, persistent bounce-loop kernel, vectorised histogram
splats); this package is its Python host side.
"""
from .scene import Material, Recorder, RenderResult, Scene, Source, Tracer, make_params  # noqa: F401

__all__ = ["Material", "Recorder", "RenderResult", "Scene", "Source", "Tracer", "make_params"]
