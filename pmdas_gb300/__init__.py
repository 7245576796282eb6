"""pmdas_gb300 — GB300-native MDAS (multidimensional adaptive sampling).

The compute path is libpmdas_gb300.so (hand-written sm_103a CUDA kernels
behind the C ABI of include/mdas.h); this package is its host-side mirror of
the reference's ``mdas::KDGrid`` interface.
"""
from ._native import (ARITH_IEEE, ARITH_REFERENCE, MdasError, SCENE_DIRECT_LIGHT, SCENE_DISCS_DOF,
                      SCENE_DISCS_MB, SCENE_DISCS_MBDOF, load)
from .kdgrid import (Batch, KDGrid, Scene, mlp_adam, mlp_forward, mlp_gradients, morton_decode, morton_encode, morton_key_bits,
                     radix_sort_pairs, read_image, render, render_graph, render_host, save_image)
from .workloads import WORKLOADS, Workload

__all__ = ["Batch", "KDGrid", "Scene", "mlp_adam", "mlp_forward", "mlp_gradients", "morton_decode", "morton_encode",
           "morton_key_bits", "radix_sort_pairs", "read_image", "render", "render_graph", "render_host", "save_image",
           "load", "MdasError",
           "ARITH_REFERENCE", "ARITH_IEEE", "SCENE_DISCS_MB", "SCENE_DISCS_DOF", "SCENE_DISCS_MBDOF",
           "SCENE_DIRECT_LIGHT", "WORKLOADS", "Workload"]
