"""katric_gb300: exact local triangle counting on one GB300 (sm_103a).

The GPU form of KaTric's shared-memory counting path: orientation by (degree, id),
per-vertex out-lists, set intersection, with a u64 total and u64 per-vertex counts.
The compute path is libktri.so (include/ktri.h); this package is its host mirror.
"""
from ._native import KtriError, load
from .counter import (Config, LocalStatistics, Plan, Statistics, TriangleCounter, default_counter, intersection,
                      preprocessing, run_shmem)
from .graph import Batch, Graph, generate
from .serve import Server

__all__ = [
    "Batch", "Config", "Graph", "Plan", "KtriError", "LocalStatistics", "Statistics", "TriangleCounter", "default_counter",
    "generate", "intersection", "load", "preprocessing", "run_shmem", "Server",
]
