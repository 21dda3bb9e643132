"""GPU: the coarse segment of a pass (preparation through the read-back of
the fine job lists) captured as a CUDA graph and replayed (GBR_OPT_GRAPH).
A worker calls the same batch size four times: the first runs directly, the
second is captured and launched, the last two replay the graph; a settings
change invalidates the graph (captured again).  Results equal those of a
worker that launches directly: poses and significant counts bit for bit,
PMAX to the atomic-order spread; the stage times stay measured (the graph
records the stage events)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [1, 0])
def test_graph_replay_equals_direct(precision):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from relion_gb300 import datagen
    from relion_gb300.estep import STAGES, MlDeviceBundle, MlOptimiserCuda
    ds = datagen.Dataset("cfg0_box64", seed=44, n_particles=16, healpix_order=2, psi_step=15.0)
    batches = [ds.particles(0, 8), ds.particles(8, 8)]

    def worker(graph):
        b = MlDeviceBundle(ds.model(precision=precision), device=0)
        b.setup_projector(0, ds.ref["data"], ds.ref["yinit"], ds.ref["zinit"], ds.ref["r_max"], ds.ref["pad"])
        return b, MlOptimiserCuda(b, graph=graph)

    bd, wd = worker(0)
    bg, wg = worker(1)
    seq = [0, 1, 0, 1]
    for i in seq:
        want = wd.do_expectation_some_particles(batches[i])
        t0 = wg.stage_times().copy()
        got = wg.do_expectation_some_particles(batches[i])
        dt = wg.stage_times() - t0
        for k in ("rot", "tilt", "psi", "xoff", "yoff", "nr_sign"):
            np.testing.assert_array_equal(got[k], want[k], err_msg=k)
        np.testing.assert_allclose(got["pmax"], want["pmax"], rtol=1e-6)
        for st in ("prep", "norm_gemm", "cross_gemm", "weights_coarse", "sig_jobs"):
            assert dt[STAGES.index(st)] > 0, st
    assert wg.graph_stats() == (1, 2)
    assert wd.graph_stats() == (0, 0)
    # a settings change: the graph is not replayed; captured again on the
    # second call after it
    wg.set_option("cand_cap", 1 << 15)
    wd.set_option("cand_cap", 1 << 15)
    for i in (0, 1, 0):
        want = wd.do_expectation_some_particles(batches[i])
        got = wg.do_expectation_some_particles(batches[i])
        np.testing.assert_array_equal(got["nr_sign"], want["nr_sign"])
    assert wg.graph_stats() == (2, 3)
    for w, b in ((wd, bd), (wg, bg)):
        w.close()
    ws_d, ws_g = bd.get_wsum(), bg.get_wsum()
    np.testing.assert_allclose(ws_g["sigma2_noise"], ws_d["sigma2_noise"], rtol=1e-6)
    bd.close()
    bg.close()
