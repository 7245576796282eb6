"""The adaptive pass that allocates nothing (mdas_adaptive_sampling_static),
checked against the grid's own pass (mdas_adaptive_sampling) on two passes in a
row, for every point dimension (3..6) and on states of several 1024-leaf tiles.

Who uses it: callers that cannot allocate device memory at the moment they
sample — a plugin host that hands out all device memory up front, a process
whose device memory belongs to another framework's caching allocator, or a
frame-paced renderer for which cudaMalloc/cudaFree inside a frame cost too much.
They keep the sampler state in buffers they allocated themselves, in the
reference's layout, and the pass keeps its scratch in a fixed array inside the
library.  Its results must be exactly those of the grid's pass.

This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import pmdas_gb300 as P
from pmdas_gb300 import _native as N

pytestmark = pytest.mark.gpu


# (dim, scene kind, width, height, extraImgBits, candidates): every state spans
# 16 to 32 tiles of 1024 leaves, so the cross-tile prefix of the scan is
# exercised in each dimension
CASES = {
    "mb3d": (3, P.SCENE_DISCS_MB, 128, 96, 6, 4),
    "dof4d": (4, P.SCENE_DISCS_DOF, 128, 96, 5, 4),
    "mbdof5d": (5, P.SCENE_DISCS_MBDOF, 96, 64, 5, 3),
    "mbdof6d": (6, P.SCENE_DISCS_MBDOF, 64, 64, 4, 2),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_static_pass_equals_grid_pass_two_calls(cuda, case):
    import torch
    D, kind, W, H, eib, cand = CASES[case]
    bpd, alpha = 1, 0.25
    L0 = (1 << (bpd * D)) << (2 * eib)
    maxSamples = 12 * L0
    nodeCap = 2 * maxSamples - 1  # what the reference allocates for leaves
    assert L0 >= 16 * 1024
    grid = P.KDGrid(D, maxSamples, cand, bpd, eib, alpha, W, H)  # reference arithmetic, as the static pass
    scene = P.Scene(kind, 3, 64, W, H, W, H)
    grid.InitialSampling()
    scene.evaluate(grid, 0, grid.GetNumberOfSamples())

    # the caller's own buffers, allocated once, in the reference's layout
    coords = torch.zeros(maxSamples * D, dtype=torch.float32, device="cuda")
    nodes = torch.zeros(nodeCap * 4, dtype=torch.int32, device="cuda")
    boxes = torch.zeros(nodeCap * 2 * D, dtype=torch.float32, device="cuda")
    errors = torch.zeros(nodeCap, dtype=torch.float32, device="cuda")
    seeds = torch.zeros(nodeCap, dtype=torch.int32, device="cuda")
    lib = N.load()

    for call in range(2):
        grid.ComputeErrors()
        gError = grid.GetGError()
        st = grid.dump_state()  # the state both passes start from
        n0, l0 = st["N"], st["L"]
        coords[: n0 * D].copy_(torch.from_numpy(st["coords"].ravel()))
        nodes[: l0 * 4].copy_(torch.from_numpy(st["nodes"].ravel()))
        boxes[: l0 * 2 * D].copy_(torch.from_numpy(st["boxes"].ravel()))
        errors[:l0].copy_(torch.from_numpy(st["errors"]))
        seeds.zero_()  # slots past the leaves hold no seed, as in the reference
        seeds[:l0].copy_(torch.from_numpy(st["seeds"].view(np.int32)))
        torch.cuda.synchronize()

        newSamples, newNodes = C.c_int(-1), C.c_int(-1)
        rc = lib.mdas_adaptive_sampling_static(D, n0, l0, cand, alpha, gError, maxSamples, nodeCap,
                                               coords.data_ptr(), nodes.data_ptr(), boxes.data_ptr(),
                                               errors.data_ptr(), seeds.data_ptr(), C.byref(newSamples),
                                               C.byref(newNodes), None)
        assert rc == N.MDAS_OK, N.status_string(rc)

        grid.AdaptiveSampling()  # the existing entry point, same state
        want = grid.dump_state()
        n1, l1 = want["N"], want["L"]
        assert (n0 + newSamples.value, l0 + newNodes.value) == (n1, l1), call
        assert newSamples.value > 0 and newNodes.value > 0
        got_coords = coords[: n1 * D].cpu().numpy().reshape(n1, D)
        got_nodes = nodes[: l1 * 4].cpu().numpy().reshape(l1, 4)
        got_boxes = boxes[: l1 * 2 * D].cpu().numpy().reshape(l1, 2 * D)
        # exact: same arithmetic, same slot order
        np.testing.assert_array_equal(got_coords.view(np.uint32), want["coords"].view(np.uint32))
        np.testing.assert_array_equal(got_nodes, want["nodes"])
        np.testing.assert_array_equal(got_boxes.view(np.uint32), want["boxes"].view(np.uint32))
        np.testing.assert_array_equal(errors[:l1].cpu().numpy(), want["errors"])
        np.testing.assert_array_equal(seeds[:l1].cpu().numpy().view(np.uint32), want["seeds"])

        n, nn = grid.GetNumberOfSamples(), grid.GetNewSamples()
        scene.evaluate(grid, n - nn, nn)  # the integrand for the new samples, before the next pass


def test_static_pass_rejects_sizes_beyond_its_scratch(cuda):
    lib = N.load()
    a, b = C.c_int(), C.c_int()
    dummy = 1 << 20  # never dereferenced: the size check comes first
    rc = lib.mdas_adaptive_sampling_static(4, 0, (1 << 22) + 1, 4, 0.25, 1.0, 1 << 29, 1 << 29,
                                           dummy, dummy, dummy, dummy, dummy, C.byref(a), C.byref(b), None)
    assert rc == N.MDAS_ERR_INVALID
    rc = lib.mdas_adaptive_sampling_static(4, 100, 100, 4, 0.25, 1.0, 150, 1000, dummy, dummy, dummy, dummy, dummy,
                                           C.byref(a), C.byref(b), None)
    assert rc == N.MDAS_ERR_CAPACITY
