"""Generate the golden vectors of the reference's own MDAS kernels.

Runs the reference's CUDA sampler (SDK/lib/mdas/kdgrid.cu, built into
oracle/_ref by oracle/build.py) on a GPU for a few small grids of every point
dimension, and stores, per case:

  * the initial sampling state (InitialSampling),
  * for each pass: the state before it (with the integrand's values), the
    errors and g_error of ComputeErrors, and the state after AdaptiveSampling,
  * Integrate / ConvertToBytes / SamplingDensity of the final state.

Sample values come from this library's analytic integrand evaluated on the
reference's own buffers.  The CPU tests (tests/test_golden.py) check the
oracle against these files.

Usage (on a machine with a GPU and oracle/_ref built):
    python tests/golden/make_golden.py --out tests/golden
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

# name: (scene kind, dim, W, H, bitsPerDim, extraImgBits, scaleFactor, alpha, candidatesNum, seed, prims, passes)
CASES = {
    "d3_mb": (0, 3, 16, 16, 1, 2, 1.0, 0.25, 4, 0, 16, 3),
    "d4_dof": (1, 4, 16, 12, 1, 1, 1.0, 0.25, 4, 1, 32, 3),
    "d5_mbdof": (2, 5, 12, 12, 1, 1, 1.0, 0.0625, 3, 2, 32, 3),
    "d6_mbdof": (2, 6, 8, 8, 1, 0, 1.0, 0.25, 5, 3, 16, 3),
    "d4_dl": (3, 4, 20, 12, 0, 3, 0.5, 0.015625, 4, 4, 4, 3),
    "d4_dof_big": (1, 4, 64, 64, 1, 4, 1.0, 0.25, 4, 5, 64, 2),
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(ROOT, "tests", "golden"))
    args = ap.parse_args()
    import torch

    import pmdas_gb300 as P
    from oracle import pyoracle as O

    assert O.RefGrid.available(), "oracle/_ref/libmdas_ref.so is not built"
    lib = O.RefGrid.lib()
    os.makedirs(args.out, exist_ok=True)
    for name, (kind, D, W, H, bpd, eib, sf, alpha, cand, seed, prims, passes) in CASES.items():
        sx, sy = sf * W, sf * H
        L0 = (1 << (bpd * D)) << (2 * eib)
        ms = 4 * L0 * 4
        ref = O.RefGrid(D, ms, cand, bpd, eib, alpha, sx, sy)
        sc = P.Scene(kind, seed, prims, sx, sy, W, H)
        out = dict(params=np.array([kind, D, W, H, bpd, eib, cand, seed, prims, passes, ms], np.int64),
                   fparams=np.array([sf, alpha, sx, sy], np.float32))
        ref.initial_sampling()
        st = ref.dump_state()
        for k in ("coords", "nodes", "boxes", "errors", "seeds"):
            out[f"init_{k}"] = st[k]
        n = st["N"]
        sc.evaluate_buffers(ref.ptr(0), ref.ptr(1), D, 0, n)
        torch.cuda.synchronize()
        for p in range(passes):
            pre = ref.dump_state()
            for k in ("coords", "values", "nodes", "boxes", "errors", "seeds"):
                out[f"p{p}_pre_{k}"] = pre[k]
            g = ref.compute_errors()
            out[f"p{p}_gerr"] = np.array([g], np.float32)
            out[f"p{p}_errors"] = ref.dump_state()["errors"]
            ref.adaptive_sampling()
            post = ref.dump_state()
            for k in ("coords", "nodes", "boxes", "errors", "seeds"):
                out[f"p{p}_post_{k}"] = post[k]
            n, nn, _, _ = ref.counts()
            sc.evaluate_buffers(ref.ptr(0), ref.ptr(1), D, n - nn, nn)
            torch.cuda.synchronize()
        fin = ref.dump_state()
        for k in ("coords", "values", "nodes", "boxes", "errors", "seeds"):
            out[f"final_{k}"] = fin[k]
        px = torch.zeros(H, W, 4, device="cuda")
        assert lib.ref_integrate(ref.h, px.data_ptr(), W, H) == 0
        b = torch.zeros(H, W, 4, dtype=torch.uint8, device="cuda")
        assert lib.ref_convert_to_bytes(ref.h, px.data_ptr(), b.data_ptr(), W, H) == 0
        d = np.zeros((H, W, 4), np.float32)
        lib.ref_sampling_density(ref.h, d.ctypes.data, W, H)
        out["final_pixels"] = px.cpu().numpy()
        out["final_bytes"] = b.cpu().numpy()
        out["final_density"] = d
        ref.close()
        path = os.path.join(args.out, f"ref_{name}.npz")
        np.savez_compressed(path, **out)
        print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
