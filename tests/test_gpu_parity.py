"""GPU parity of the CUDA kernels (through the C ABI) against
  * the CPU oracle, bit for bit, in the strict-IEEE build (MDAS_ARITH_IEEE);
  * the reference's own CUDA kernels (oracle/_ref), bit for bit per pass from
    the same state, in the reference-arithmetic build (MDAS_ARITH_REFERENCE).
Images are compared within 1e-5 relative (float atomics sum in any order)."""
import ctypes as C

import numpy as np
import pytest

import pmdas_gb300 as P
from pmdas_gb300 import _native as N
from oracle import pyoracle as O
from tests.parity import assert_pass_equivalent, assert_states_equal, rel_close

pytestmark = pytest.mark.gpu

# (scene kind, dim, W, H, spp, bitsPerDim, extraImgBits, scaleFactor, alpha, candidatesNum, seed, prims)
CASES = {
    "mb3d": (P.SCENE_DISCS_MB, 3, 96, 80, 8, 1, 4, 1.0, 0.25, 4, 0, 64),
    "dof4d": (P.SCENE_DISCS_DOF, 4, 128, 128, 16, 1, 5, 1.0, 0.25, 4, 1, 256),
    "mbdof5d": (P.SCENE_DISCS_MBDOF, 5, 120, 68, 12, 1, 3, 1.0, 0.0625, 4, 2, 128),
    "dl4d": (P.SCENE_DIRECT_LIGHT, 4, 160, 90, 10, 0, 6, 0.5, 0.015625, 3, 3, 4),
    "mbdof6d": (P.SCENE_DISCS_MBDOF, 6, 64, 64, 8, 1, 2, 1.0, 0.25, 5, 4, 64),
}


def make(case, arith, maxSamples=None):
    kind, D, W, H, spp, bpd, eib, sf, alpha, cand, seed, prims = CASES[case]
    sx, sy = sf * W, sf * H
    budget = int(spp * W * H)
    ms = maxSamples or 2 * budget + 4 * ((1 << (bpd * D)) << (2 * eib))
    g = P.KDGrid(D, ms, cand, bpd, eib, alpha, sx, sy, arith=arith)
    sc = P.Scene(kind, seed, prims, sx, sy, W, H)
    o = O.OracleGrid(D, ms, cand, bpd, eib, alpha, sx, sy)
    return g, sc, o, dict(D=D, W=W, H=H, budget=budget, sx=sx, sy=sy)


@pytest.mark.parametrize("case", list(CASES))
def test_ieee_build_matches_oracle_every_pass(cuda, case):
    g, sc, o, p = make(case, P.ARITH_IEEE)
    desc = sc.export()
    g.InitialSampling()
    o.initial_sampling()
    assert_states_equal(g.dump_state(), o.dump_state(), what="initial sampling")
    sc.evaluate(g, 0, g.GetNumberOfSamples())
    o.evaluate(desc, 0, o.N)
    a = g.dump_state()
    assert np.array_equal(a["values"].view(np.uint32), o.values[:o.N].view(np.uint32)), "integrand values"
    passes = 0
    while g.GetNumberOfSamples() < p["budget"]:
        g.SamplingPass()
        o.sampling_pass()
        assert g.GetGError() == o.gerr
        n, nn = g.GetNumberOfSamples(), g.GetNewSamples()
        sc.evaluate(g, n - nn, nn)
        o.evaluate(desc, o.N - o.newN, o.newN)
        assert_states_equal(g.dump_state(), o.dump_state(), keys=("coords", "values", "nodes", "boxes", "errors",
                                                                   "seeds"), what=f"pass {passes}")
        passes += 1
    assert passes >= 2
    assert g.Validate() and o.validate() == 0
    import torch
    px = torch.zeros(p["H"], p["W"], 4, device="cuda")
    g.Integrate(px, p["W"], p["H"])
    img = px.cpu().numpy()
    ref = o.integrate(p["W"], p["H"])
    ok, worst = rel_close(img, ref)
    assert ok, worst
    # bytes of the same float image are bit-exact
    b = torch.zeros(p["H"], p["W"], 4, dtype=torch.uint8, device="cuda")
    px.copy_(torch.from_numpy(ref).cuda())
    g.ConvertToBytes(px, b, p["W"], p["H"])
    assert np.array_equal(b.cpu().numpy(), O.convert_to_bytes(ref))
    # sampling density (host code in the reference: IEEE in both builds)
    dens = np.zeros((p["H"], p["W"], 4), np.float32)
    g.SamplingDensity(dens, p["W"], p["H"])
    assert np.array_equal(dens, o.sampling_density(p["W"], p["H"]))


def test_render_loop_matches_oracle(cuda):
    """mdas_render (the whole budget loop behind one call) == the oracle's loop."""
    import torch
    g, sc, o, p = make("dof4d", P.ARITH_IEEE)
    px = torch.zeros(p["H"], p["W"], 4, device="cuda")
    st = P.render(g, sc, p["budget"], px, p["W"], p["H"])
    img, n, l, passes, _, _ = O.render(p["D"], 1, 5, 4, 0.25, p["sx"], p["sy"], p["budget"], g.GetMaxSamples(),
                                       sc.export(), p["W"], p["H"], threads=4)
    assert (st.numberOfSamples, st.numberOfNodes, st.passes) == (n, l, passes)
    ok, worst = rel_close(px.cpu().numpy(), img)
    assert ok, worst
    # and the host-buffer entry point gives the same image
    host = np.zeros((p["H"], p["W"], 4), np.float32)
    st2 = P.render_host(g, sc, p["budget"], host, p["W"], p["H"], host_prims=sc.export().prims)
    assert st2.numberOfSamples == n
    ok, worst = rel_close(host, img)
    assert ok, worst


@pytest.mark.parametrize("arith", [P.ARITH_REFERENCE, P.ARITH_IEEE])
@pytest.mark.parametrize("case", ["mb3d", "dof4d", "mbdof5d"])
def test_render_graph_equals_host_loop(cuda, arith, case):
    """The device-side loop (one CUDA graph) leaves exactly the state of the
    host-driven loop, and a second launch of the cached graph does too."""
    import torch
    g1, sc, _, p = make(case, arith)
    g2 = P.KDGrid(p["D"], g1.GetMaxSamples(), CASES[case][9], CASES[case][5], CASES[case][6], CASES[case][8],
                  p["sx"], p["sy"], arith=arith)
    px1 = torch.zeros(p["H"], p["W"], 4, device="cuda")
    px2 = torch.zeros(p["H"], p["W"], 4, device="cuda")
    st1 = P.render(g1, sc, p["budget"], px1, p["W"], p["H"])
    a = g1.dump_state()
    for launch in range(2):
        st2 = P.render_graph(g2, sc, p["budget"], px2, p["W"], p["H"])
        assert (st2.numberOfSamples, st2.numberOfNodes, st2.passes) == \
            (st1.numberOfSamples, st1.numberOfNodes, st1.passes), launch
        assert_states_equal(g2.dump_state(), a, keys=("coords", "values", "nodes", "boxes", "errors", "seeds"),
                            what=f"graph launch {launch}")
        ok, worst = rel_close(px2.cpu().numpy(), px1.cpu().numpy())
        assert ok, worst
    assert g2.Validate()


@pytest.mark.parametrize("arith", [P.ARITH_REFERENCE, P.ARITH_IEEE])
def test_batch_equals_single_renders(cuda, arith):
    """A batch of images of different dimension, size and budget (one launch per
    stage and dimension, device-side loop) leaves every image exactly as its
    own render would; a second render and a retuned graph do too."""
    import torch
    specs = [  # (kind, D, W, H, spp, bpd, eib, alpha, cand, seed, prims)
        (P.SCENE_DISCS_MB, 3, 64, 48, 8, 1, 3, 0.25, 4, 11, 32),
        (P.SCENE_DISCS_DOF, 4, 96, 64, 16, 1, 3, 0.25, 4, 12, 64),
        (P.SCENE_DISCS_MBDOF, 5, 40, 40, 12, 1, 2, 0.0625, 3, 13, 32),
        (P.SCENE_DISCS_MB, 3, 128, 128, 4, 1, 4, 0.5, 2, 14, 64),
        (P.SCENE_DIRECT_LIGHT, 4, 80, 60, 32, 0, 5, 0.015625, 4, 15, 4),
        (P.SCENE_DISCS_DOF, 4, 32, 32, 2, 1, 3, 0.25, 4, 16, 16),  # budget below the initial grid: no pass
        # a larger image (1280 x 1024) beside the small ones
        (P.SCENE_DISCS_DOF, 4, 1280, 1024, 1, 0, 7, 0.25, 4, 17, 32),
    ]
    grids, scenes, pix, budgets, singles = [], [], [], [], []
    for kind, D, W, H, spp, bpd, eib, alpha, cand, seed, prims in specs:
        budget = spp * W * H
        ms = 2 * budget + 8 * ((1 << (bpd * D)) << (2 * eib))
        sc = P.Scene(kind, seed, prims, W, H, W, H)
        ref = P.KDGrid(D, ms, cand, bpd, eib, alpha, W, H, arith=arith)
        rpx = torch.zeros(H, W, 4, device="cuda")
        st = P.render(ref, sc, budget, rpx, W, H)
        singles.append((ref.dump_state(), rpx.cpu().numpy(), st.passes))
        grids.append(P.KDGrid(D, ms, cand, bpd, eib, alpha, W, H, arith=arith))
        scenes.append(sc)
        pix.append(torch.zeros(H, W, 4, device="cuda"))
        budgets.append(budget)
    batch = P.Batch(grids, scenes, budgets, pix, [sp[2] for sp in specs], [sp[3] for sp in specs])
    for rnd in range(5):
        if rnd == 2:
            batch.set_tuning([2, 3, 1, 5])
        if rnd == 3:  # decide tiles of 1024 leaves: same results
            batch.set_tiling([3, 2, 2, 4], 1024)
        # the last round with the pass loop on the host
        stats = batch.render_stepped() if rnd == 4 else batch.render()
        for i, (want, img, passes) in enumerate(singles):
            assert stats[i].passes == passes, (rnd, i)
            assert_states_equal(grids[i].dump_state(), want,
                                keys=("coords", "values", "nodes", "boxes", "errors", "seeds"), what=f"image {i}")
            ok, worst = rel_close(pix[i].cpu().numpy(), img)
            assert ok, (i, worst)
    assert singles[-2][2] == 0 and singles[0][2] > 0 and singles[-1][2] > 0
    batch.close()


def test_batch_ieee_matches_oracle_directly(cuda):
    """A strict-IEEE batch of three images of different dimension, compared with
    the CPU oracle's own budget loop for each image (not only with single GPU
    renders): the whole final state bit for bit and the image within 1e-5."""
    import torch
    specs = [  # (kind, D, W, H, spp, bpd, eib, alpha, cand, seed, prims)
        (P.SCENE_DISCS_MB, 3, 48, 32, 8, 1, 3, 0.25, 4, 21, 32),
        (P.SCENE_DISCS_DOF, 4, 64, 48, 12, 1, 3, 0.25, 4, 22, 48),
        (P.SCENE_DISCS_MBDOF, 5, 32, 32, 10, 1, 2, 0.0625, 3, 23, 32),
    ]
    grids, scenes, pix, budgets = [], [], [], []
    for kind, D, W, H, spp, bpd, eib, alpha, cand, seed, prims in specs:
        budget = spp * W * H
        ms = 2 * budget + 8 * ((1 << (bpd * D)) << (2 * eib))
        scenes.append(P.Scene(kind, seed, prims, W, H, W, H))
        grids.append(P.KDGrid(D, ms, cand, bpd, eib, alpha, W, H, arith=P.ARITH_IEEE))
        pix.append(torch.zeros(H, W, 4, device="cuda"))
        budgets.append(budget)
    batch = P.Batch(grids, scenes, budgets, pix, [sp[2] for sp in specs], [sp[3] for sp in specs])
    stats = batch.render()
    for i, (kind, D, W, H, spp, bpd, eib, alpha, cand, seed, prims) in enumerate(specs):
        ms = grids[i].GetMaxSamples()
        o = O.OracleGrid(D, ms, cand, bpd, eib, alpha, W, H)
        desc = scenes[i].export()
        o.initial_sampling()
        o.evaluate(desc, 0, o.N)
        passes = 0
        while o.N < budgets[i] and o.N + o.L <= ms:
            o.sampling_pass()
            o.evaluate(desc, o.N - o.newN, o.newN)
            passes += 1
        assert stats[i].passes == passes and passes > 0, (i, stats[i].passes, passes)
        assert_states_equal(grids[i].dump_state(), o.dump_state(),
                            keys=("coords", "values", "nodes", "boxes", "errors", "seeds"), what=f"image {i}")
        ok, worst = rel_close(pix[i].cpu().numpy(), o.integrate(W, H))
        assert ok, (i, worst)
    batch.close()


def test_reference_build_close_to_oracle(cuda):
    """The fast-math build differs from IEEE only in the last bits of divisions,
    square roots and powf: same initial grid (power-of-two extents), errors within
    a few ulps, and the same leaf decisions except for near-ties."""
    g, sc, o, p = make("dof4d", P.ARITH_REFERENCE)
    desc = sc.export()
    g.InitialSampling()
    o.initial_sampling()
    assert_states_equal(g.dump_state(), o.dump_state(), what="initial sampling")
    sc.evaluate(g, 0, g.GetNumberOfSamples())
    s0 = g.dump_state()
    o.load_state(s0)
    g.ComputeErrors()
    o.compute_errors()
    a = g.dump_state()
    np.testing.assert_allclose(a["errors"], o.errors[:o.L], rtol=2e-6)
    g.AdaptiveSampling()
    o.adaptive_sampling()
    a = g.dump_state()
    same = np.mean(a["seeds"][:s0["L"]] == o.seeds[:s0["L"]])
    assert same > 0.999
    assert abs(a["N"] - o.N) <= 0.001 * s0["L"]


@pytest.fixture(scope="module")
def refgrid_cls():
    if not O.RefGrid.available():
        pytest.skip("reference harness oracle/_ref not built (needs the reference checkout at build time)")
    return O.RefGrid


@pytest.mark.parametrize("case", ["mb3d", "dof4d", "mbdof5d", "dl4d", "mbdof6d"])
def test_reference_build_matches_reference_kernels(cuda, refgrid_cls, case):
    import torch
    kind, D, W, H, spp, bpd, eib, sf, alpha, cand, seed, prims = CASES[case]
    g, sc, _, p = make(case, P.ARITH_REFERENCE)
    ms = g.GetMaxSamples()
    ref = refgrid_cls(D, ms, cand, bpd, eib, alpha, p["sx"], p["sy"])
    try:
        g.InitialSampling()
        ref.initial_sampling()
        assert_states_equal(g.dump_state(), ref.dump_state(), what="initial sampling vs reference")
        sc.evaluate(g, 0, g.GetNumberOfSamples())
        for k in range(5):
            if g.GetNumberOfSamples() >= p["budget"]:
                break
            s0 = g.dump_state()
            ref.load_state(s0)
            gref = ref.compute_errors()
            g.ComputeErrors()
            assert g.GetGError() == gref, (k, g.GetGError(), gref)
            after_err = g.dump_state()
            rs = ref.dump_state()
            assert np.array_equal(after_err["errors"].view(np.uint32), rs["errors"].view(np.uint32)), k
            ref.adaptive_sampling()
            g.AdaptiveSampling()
            assert_pass_equivalent(s0, g.dump_state(), ref.dump_state(), D, what=f"{case} pass {k}")
            n, nn = g.GetNumberOfSamples(), g.GetNewSamples()
            sc.evaluate(g, n - nn, nn)
        # reconstruction from the same state: within 1e-5 (summation order)
        st = g.dump_state()
        ref.load_state(st)
        px = torch.zeros(H, W, 4, device="cuda")
        g.Integrate(px, W, H)
        rpx = torch.zeros(H, W, 4, device="cuda")
        assert refgrid_cls.lib().ref_integrate(ref.h, rpx.data_ptr(), W, H) == 0
        ok, worst = rel_close(px.cpu().numpy(), rpx.cpu().numpy())
        assert ok, worst
        # bytes from the same float image: bit-exact
        b = torch.zeros(H, W, 4, dtype=torch.uint8, device="cuda")
        rb = torch.zeros(H, W, 4, dtype=torch.uint8, device="cuda")
        g.ConvertToBytes(rpx, b, W, H)
        assert refgrid_cls.lib().ref_convert_to_bytes(ref.h, rpx.data_ptr(), rb.data_ptr(), W, H) == 0
        assert torch.equal(b, rb)
        # sampling density (host loop in the reference)
        d = np.zeros((H, W, 4), np.float32)
        rd = np.zeros((H, W, 4), np.float32)
        g.SamplingDensity(d, W, H)
        refgrid_cls.lib().ref_sampling_density(ref.h, rd.ctypes.data, W, H)
        assert np.array_equal(d, rd)
    finally:
        ref.close()


def test_reference_image_and_rel_mse(cuda):
    """The FP64 reference image converges, and an MDAS image at 16 spp is close to it."""
    import torch
    from tests.parity import rel_mse
    g, sc, _, p = make("dof4d", P.ARITH_REFERENCE)
    W, H = p["W"], p["H"]
    ref = sc.reference_image(W, H, spp=4096).cpu().numpy()
    ref_lo = sc.reference_image(W, H, spp=1024, seed=7).cpu().numpy()
    assert np.all(np.isfinite(ref)) and ref.min() >= 0.0 and ref.max() <= 1.0 + 1e-12
    assert rel_mse(ref_lo, ref) < 5e-4  # Monte Carlo noise of the 1024-spp image at disc edges
    px = torch.zeros(H, W, 4, device="cuda")
    P.render(g, sc, p["budget"], px, W, H)
    img = px[..., :3].cpu().numpy()
    e = rel_mse(img, ref)
    assert e < 2e-2, e
    # a flat image of the mean colour is far worse: the sampler resolves the scene
    flat = np.broadcast_to(ref.mean(axis=(0, 1)), ref.shape)
    assert rel_mse(flat, ref) > 10 * e


# ---- edge cases ------------------------------------------------------------------
def test_capacity_is_an_error_not_an_overrun(cuda):
    # initial grid alone (128 leaves, 512 samples) does not fit
    g = P.KDGrid(3, 500, 4, 1, 2, 0.25, 16, 16)
    with pytest.raises(N.MdasError) as e:
        g.InitialSampling()
    assert e.value.status == N.MDAS_ERR_CAPACITY
    # initial grid fits (512 samples, 128 leaves) but a pass could add 128 more
    g = P.KDGrid(3, 600, 4, 1, 2, 0.25, 16, 16)
    g.InitialSampling()
    with pytest.raises(N.MdasError) as e:
        g.SamplingPass()
    assert e.value.status == N.MDAS_ERR_CAPACITY
    assert g.GetNumberOfSamples() == 512


def test_call_order_checked(cuda):
    g = P.KDGrid(4, 10000, 4, 1, 1, 0.25, 8, 8)
    with pytest.raises(N.MdasError) as e:
        g.SamplingPass()
    assert e.value.status == N.MDAS_ERR_STATE


@pytest.mark.parametrize("arith", [P.ARITH_IEEE, P.ARITH_REFERENCE])
def test_ragged_tiles_and_parameter_extremes(cuda, arith):
    """Leaf counts that are not multiples of the 256-leaf tile, 1 and 8 candidates,
    all-zero and constant values, and alphas that select everything / almost nothing."""
    for D, bpd, eib, cand, alpha in ((3, 1, 0, 1, 0.25), (5, 1, 1, 8, 4.0), (4, 1, 2, 2, 1e-3), (6, 0, 3, 4, 0.5)):
        sx = sy = 10.0
        ms = 200000
        g = P.KDGrid(D, ms, cand, bpd, eib, alpha, sx, sy, arith=arith)
        o = O.OracleGrid(D, ms, cand, bpd, eib, alpha, sx, sy)
        g.InitialSampling()
        o.initial_sampling()
        rng = np.random.default_rng(D)
        for k in range(5):
            st = g.dump_state()
            vals = rng.random((st["N"], 3), dtype=np.float32)
            if k == 1:
                vals[:] = 0.0
            if k == 2:
                vals[:] = 0.25
            st["values"] = vals
            g.load_state(st)
            o.load_state(st)
            g.SamplingPass()
            o.sampling_pass()
            if arith == P.ARITH_IEEE:
                assert_states_equal(g.dump_state(), o.dump_state(), what=f"D{D} pass {k}")
            assert g.Validate()


def test_dump_load_roundtrip_and_log(cuda, tmp_path):
    logp = tmp_path / "run.exr.log"
    g = P.KDGrid(4, 500000, 4, 1, 3, 0.25, 64, 64, log=str(logp))
    sc = P.Scene(P.SCENE_DISCS_DOF, 9, 64, 64, 64, 64, 64)
    g.InitialSampling()
    sc.evaluate(g, 0, g.GetNumberOfSamples())
    g.SamplingPass()
    st = g.dump_state()
    h = P.KDGrid(4, 500000, 4, 1, 3, 0.25, 64, 64)
    h.load_state(st)
    assert_states_equal(h.dump_state(), st, keys=("coords", "values", "nodes", "boxes", "errors", "seeds"))
    import torch
    px = torch.zeros(64, 64, 4, device="cuda")
    g.Integrate(px, 64, 64)
    g.close()
    text = logp.read_text().split("\n")
    for key in ("INITIAL SAMPLES", "INITIAL SAMPLING TIME", "COMPUTE ERRORS TIME", "SAMPLES",
                "ADAPTIVE SAMPLING TIME", "TOTAL SAMPLES", "INTEGRATE TIME"):
        assert key in text, key
    assert int(text[text.index("INITIAL SAMPLES") + 1]) == 4 * (1 << 10)


def test_device_views_and_stream(cuda):
    import torch
    s = torch.cuda.Stream()
    g = P.KDGrid(3, 100000, 4, 1, 3, 0.25, 32, 32, stream=s.cuda_stream)
    with torch.cuda.stream(s):
        g.InitialSampling()
        c = g.GetSampleCoordinates()
        v = g.GetSampleValues()
        v.copy_(c[:, :3] / 32.0)  # a caller-side integrand writing in place
    s.synchronize()
    assert c.shape == (g.GetNumberOfSamples(), 3)
    st = g.dump_state()
    np.testing.assert_allclose(st["values"][:, 0], st["coords"][:, 0] / 32.0, rtol=1e-6)
    g.SamplingPass()
    assert g.GetNewSamples() > 0 and g.Validate()
    assert g.launch_count() >= 4


# ---- the dof1024 workload at full size (4-D, 1024x1024, 16 spp) ---------------------
def _full_size(arith, name="dof1024"):
    from pmdas_gb300.workloads import WORKLOADS
    w = WORKLOADS[name]
    g = P.KDGrid(w.dim, w.maxSamples, w.candidatesNum, w.bitsPerDim, w.extraImgBits, w.alpha, w.scaleX, w.scaleY,
                 arith=arith)
    sc = P.Scene(w.scene_kind, w.scene_seed, w.scene_count, w.scaleX, w.scaleY, w.width, w.height)
    return w, g, sc


@pytest.mark.slow
def test_full_size_graph_equals_host_loop_and_partitions(cuda):
    """16.8 M samples in about 6 M leaves, checked through properties that need
    no CPU restatement: the device-side loop and the host loop end in the same
    state bit for bit, the images agree within the atomic-order tolerance, and
    the leaves partition the domain with every sample in exactly one leaf,
    inside its box."""
    torch = cuda
    w, a, sc = _full_size(P.ARITH_REFERENCE)
    _, b, _ = _full_size(P.ARITH_REFERENCE)
    pa = torch.zeros(w.height, w.width, 4, device="cuda")
    pb = torch.zeros(w.height, w.width, 4, device="cuda")
    sa = P.render_graph(a, sc, w.budget, pa, w.width, w.height)
    sb = P.render(b, sc, w.budget, pb, w.width, w.height)
    assert (sa.numberOfSamples, sa.numberOfNodes, sa.passes) == (sb.numberOfSamples, sb.numberOfNodes, sb.passes)
    assert sa.numberOfSamples >= w.budget and sa.numberOfNodes > 4_000_000
    assert_states_equal(a.dump_state(), b.dump_state(), keys=("coords", "values", "nodes", "boxes", "errors", "seeds"),
                        what="dof1024 graph vs host loop")
    ok, worst = rel_close(pa.cpu().numpy(), pb.cpu().numpy())
    assert ok, worst
    assert torch.isfinite(pa).all() and float(pa[..., :3].min()) >= 0.0
    assert a.Validate()


@pytest.mark.slow
@pytest.mark.parametrize("name", ["dof1024", "mbdof1080"])
def test_full_size_pass_matches_reference_kernels(cuda, refgrid_cls, name):
    """From the final state of a full-size render (dof1024: 4-D, 16.8 M samples;
    mbdof1080: 5-D, 1920x1080 at 32 spp, 66 M samples): one more errors pass
    and adaptive pass equal the reference's kernels on the same state (slot
    order canonicalised), and the reconstruction agrees within 1e-5."""
    torch = cuda
    w, g, sc = _full_size(P.ARITH_REFERENCE, name)
    px = torch.zeros(w.height, w.width, 4, device="cuda")
    P.render_graph(g, sc, w.budget, px, w.width, w.height)
    ref = refgrid_cls(w.dim, w.maxSamples, w.candidatesNum, w.bitsPerDim, w.extraImgBits, w.alpha, w.scaleX, w.scaleY)
    try:
        s0 = g.dump_state()
        ref.load_state(s0)
        rpx = torch.zeros(w.height, w.width, 4, device="cuda")
        assert refgrid_cls.lib().ref_integrate(ref.h, rpx.data_ptr(), w.width, w.height) == 0
        g.Integrate(px, w.width, w.height)
        ok, worst = rel_close(px.cpu().numpy(), rpx.cpu().numpy())
        assert ok, worst
        gref = ref.compute_errors()
        g.ComputeErrors()
        assert g.GetGError() == gref
        assert np.array_equal(g.dump_state()["errors"].view(np.uint32), ref.dump_state()["errors"].view(np.uint32))
        ref.adaptive_sampling()
        g.AdaptiveSampling()
        assert_pass_equivalent(s0, g.dump_state(), ref.dump_state(), w.dim, what=f"{name} full-size pass")
        assert g.Validate()
    finally:
        ref.close()


@pytest.mark.slow
@pytest.mark.parametrize("name", ["dof1024", "mbdof1080"])
def test_full_size_ieee_pass_matches_oracle(cuda, name):
    """The strict-IEEE build at full size: from the final state of a render,
    one more sampling pass (errors, acceptance, candidates, splits over all its
    leaves) is the CPU oracle's, bit for bit and slot for slot."""
    torch = cuda
    w, g, sc = _full_size(P.ARITH_IEEE, name)
    P.render_graph(g, sc, w.budget, torch.zeros(w.height, w.width, 4, device="cuda"), w.width, w.height)
    o = O.OracleGrid(w.dim, w.maxSamples, w.candidatesNum, w.bitsPerDim, w.extraImgBits, w.alpha, w.scaleX, w.scaleY)
    o.load_state(g.dump_state())
    g.SamplingPass()
    o.sampling_pass()
    assert g.GetGError() == o.gerr
    assert g.GetNewSamples() == o.newN > 0
    assert_states_equal(g.dump_state(), o.dump_state(), keys=("coords", "nodes", "boxes", "errors", "seeds"),
                        what=f"{name} full-size pass vs oracle")


def test_pass_accumulators_without_memsets(cuda):
    """No pass clears its accumulators with a memset: the adaptive pass's scan
    keeps them for the host and clears them for the next pass.  g_error stays
    the last errors pass's after the adaptive pass (as the reference's
    __device__ g_error does), a repeated errors pass gives the same g_error,
    and the pass tallies match the dumped state."""
    g, sc, _, c = make("dof4d", P.ARITH_REFERENCE)
    g.InitialSampling()
    sc.evaluate(g, 0, g.GetNumberOfSamples())
    for k in range(4):
        g.ComputeErrors()
        ge = g.GetGError()
        st = g.dump_state()
        assert ge == float(st["errors"].max())  # the max over every leaf
        g.ComputeErrors()  # again, no adaptive pass between: the same value
        assert g.GetGError() == ge
        L0 = g.GetNumberOfNodes()
        g.AdaptiveSampling()
        assert g.GetGError() == ge  # still this pass's after the adaptive pass
        ps = g.pass_stats()
        assert ps["selected"] == g.GetNewSamples() > 0
        assert ps["splits"] == g.GetNumberOfNodes() - L0
        # every sample coordinate the accepted leaves held was read once
        assert 0 < ps["gathered"] <= 4 * ps["selected"]
        n2, nn = g.GetNumberOfSamples(), g.GetNewSamples()
        sc.evaluate(g, n2 - nn, nn)
        if k == 0:
            assert ps["recomputed"] == L0  # the first errors pass visits every leaf
