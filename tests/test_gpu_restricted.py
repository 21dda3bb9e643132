"""GPU tests of the coarse pass restricted to orientation blocks.

gbr_expect_batch_blocks scores, for each particle, only the orientation
blocks it is given (a block: the four sibling HEALPix directions of one
parent pixel, every psi, every translation), on a tcgen05 kernel whose MMA
rows are one particle's translations; poses in other blocks get weight zero.
That is the exhaustive search under a prior that is zero outside the blocks,
so each restricted result is checked against the exhaustive precision-form
E-step (itself checked against the oracle) run with pdf_direction set to zero
outside the particle's blocks:
  * every block for every particle: identical significant counts and best
    poses, per-particle results to 1e-5, volumes to 1e-5 relative L2, and the
    stored coarse diff2 within 1e-6 relative of the exhaustive pass's;
  * one block subset for the whole batch: the same against the masked prior
    (dLL then differs by one constant, the prior's normalisation);
  * a different subset per particle (one particle exhaustive): each
    particle's results against its own masked run.
Box-64 workload, HEALPix order 2 (192 directions, 48 blocks of 4 x 48 psi),
offsets +/-4 px step 1 (49 translations).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 6


@pytest.fixture(scope="module")
def case():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from relion_gb300 import datagen
    ds = datagen.Dataset("cfg0_box64", seed=31, n_particles=N, offset_range_px=4.0, offset_step_px=1.0)
    return ds, ds.model(precision=1), ds.particles(0, N)


def _run(ds, model, batch, blocks=None, pdf_direction=None, debug=False):
    from relion_gb300.estep import MlDeviceBundle, MlOptimiserCuda
    m = dict(model)
    if pdf_direction is not None:
        m["pdf_direction"] = pdf_direction
    b = MlDeviceBundle(m, device=0)
    r = ds.ref
    b.setup_projector(0, r["data"], r["yinit"], r["zinit"], r["r_max"], r["pad"])
    nblk, dpb, rows = b.orientation_blocks()
    w = MlOptimiserCuda(b, debug=debug)
    res = w.do_expectation_some_particles(batch, blocks=blocks)
    n = len(res)
    coarse = [w.debug_fetch(0, i) for i in range(n)] if debug else None
    ws = b.get_wsum()
    vol = b.get_mdl_data(0)
    w.close()
    b.close()
    return dict(res=res, coarse=coarse, wsum=ws, vol=vol, nblk=nblk, dpb=dpb)


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def _masked_pdf(model, blocks, dpb):
    pdf = np.array(model["pdf_direction"], dtype=np.float64).copy()
    keep = np.zeros(len(pdf), bool)
    for o in blocks:
        keep[o * dpb:(o + 1) * dpb] = True
    pdf[~keep] = 0.0
    return pdf


def _same_results(a, b, dll_const=False):
    assert np.array_equal(a["nr_sign"], b["nr_sign"])
    assert np.array_equal(a["best_ihidden_over"], b["best_ihidden_over"])
    for k in ("pmax", "coarse_significant_weight", "fine_sum_weight"):
        if k != "pmax" and dll_const:
            continue  # scaled by the masked prior's normalisation
        np.testing.assert_allclose(a[k], b[k], rtol=1e-5, err_msg=k)
    d = np.asarray(a["dLL"]) - np.asarray(b["dLL"])
    if dll_const:
        assert np.ptp(d) <= 1e-4
    else:
        assert np.max(np.abs(d)) <= 1e-4


def test_all_blocks_equals_exhaustive(case):
    from relion_gb300.estep import ALL_BLOCKS
    ds, model, batch = case
    ex = _run(ds, model, batch, debug=True)
    rs = _run(ds, model, batch, blocks=np.full((N, 1), ALL_BLOCKS, np.int32), debug=True)
    _same_results(rs["res"], ex["res"])
    for k in ("sigma2_noise", "pdf_direction"):
        assert _rel(rs["wsum"][k], ex["wsum"][k]) <= 1e-5, k
    assert _rel(rs["vol"][0], ex["vol"][0]) <= 1e-5
    assert _rel(rs["vol"][1], ex["vol"][1]) <= 1e-5
    for i in range(N):
        ge, gr = ex["coarse"][i], rs["coarse"][i]
        fe = np.isfinite(ge)
        assert np.all(np.isfinite(gr[fe])), "restricted pass left out a pose the exhaustive pass stored"
        assert np.max(np.abs(gr[fe] - ge[fe]) / np.abs(ge[fe])) <= 1e-6


def test_block_subset_equals_masked_prior(case):
    ds, model, batch = case
    ex = _run(ds, model, batch)
    nblk, dpb = ex["nblk"], ex["dpb"]
    ndir = nblk * dpb
    # blocks holding each particle's exhaustive best direction plus a fixed random set
    from relion_gb300.estep import MlDeviceBundle
    b = MlDeviceBundle(model, device=0)
    npsi, ntrans, nor, ntr = b.npsi, b.ntrans, b.nover_rot, b.nover_trans
    b.close()
    best_dir = (np.asarray(ex["res"]["best_ihidden_over"]) // (nor * ntr) // ntrans // npsi) % ndir
    rng = np.random.default_rng(3)
    S = sorted(set((best_dir // dpb).tolist()) | set(rng.choice(nblk, 8, replace=False).tolist()))
    blocks = np.tile(np.array(S, np.int32), (N, 1))
    rs = _run(ds, model, batch, blocks=blocks)
    mk = _run(ds, model, batch, pdf_direction=_masked_pdf(model, S, dpb))
    _same_results(rs["res"], mk["res"], dll_const=True)
    for k in ("sigma2_noise", "pdf_direction"):
        assert _rel(rs["wsum"][k], mk["wsum"][k]) <= 1e-5, k
    assert _rel(rs["vol"][0], mk["vol"][0]) <= 1e-5
    assert _rel(rs["vol"][1], mk["vol"][1]) <= 1e-5


def test_per_particle_blocks(case):
    from relion_gb300.estep import ALL_BLOCKS
    ds, model, batch = case
    rng = np.random.default_rng(7)
    nblk = _run(ds, model, {k: (v[:1] if isinstance(v, np.ndarray) else v) for k, v in batch.items()} | {"n": 1})["nblk"]
    m = 12
    blocks = np.full((N, m), -1, np.int32)
    sets = []
    for i in range(N):
        k = int(rng.integers(3, m + 1))
        s = rng.choice(nblk, k, replace=False)
        blocks[i, :k] = s
        sets.append(sorted(s.tolist()))
    blocks[2, 0] = ALL_BLOCKS
    sets[2] = list(range(nblk))
    rs = _run(ds, model, batch, blocks=blocks)
    for i in range(N):
        one = {k: (v[i:i + 1] if isinstance(v, np.ndarray) else v) for k, v in batch.items()}
        one["n"] = 1
        mk = _run(ds, model, one, pdf_direction=_masked_pdf(model, sets[i], rs["dpb"]))
        r1 = rs["res"][i:i + 1]
        assert r1["nr_sign"][0] == mk["res"]["nr_sign"][0], i
        assert r1["best_ihidden_over"][0] == mk["res"]["best_ihidden_over"][0], i
        np.testing.assert_allclose(r1["pmax"], mk["res"]["pmax"], rtol=1e-5)
