"""GB300-native ForceAtlas2 layout engine.

A drop-in CUDA (sm_103a) backend for the forceatlas2r package's C interface
(include/fa2.h, implemented by libfa2cuda.so), plus a Python host API that
mirrors the package's R functions for the GPU paths. See layout.py.
"""
from .layout import (REPULSION_BH, REPULSION_EXACT, Graph, Layout, gpu_devices,
                     layout_forceatlas2_gpu, layout_forceatlas2_large,
                     prepare_graph)
from .batch import Batch, tune
from . import graphs

__all__ = ["gpu_devices", "layout_forceatlas2_gpu", "layout_forceatlas2_large",
           "Layout", "Graph", "prepare_graph", "graphs", "REPULSION_BH",
           "REPULSION_EXACT", "Batch", "tune"]
