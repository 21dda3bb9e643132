"""GPU-vs-oracle comparison of one E-step batch (TEST INFRASTRUCTURE ONLY).

Runs the CUDA path (libgbrelion, through relion_gb300.estep) and the CPU
oracle on the same inputs and returns error statistics for each stage.
"""
import numpy as np

from . import pyoracle

# tolerances of the plain FP32 path against the FP64 CPU oracle
TOL = dict(
    coarse_diff2_rel=1e-5,     # relative diff2
    fine_diff2_rel=1e-5,
    weight_norm_abs=1e-4,      # max normalised-weight difference
    bp_rel_l2=1e-5,            # backprojected volumes, relative L2
    argmax_agree=0.999,
)


def run_gpu(model, refs, batch, device=0, **options):
    """The CUDA E-step with the debug read-back; `options` are worker
    options (relion_gb300.estep.MlOptimiserCuda), e.g. batch_cap."""
    from relion_gb300.estep import MlDeviceBundle, MlOptimiserCuda
    b = MlDeviceBundle(model, device=device)
    for k, r in enumerate(refs):
        b.setup_projector(k, r["data"], r["yinit"], r["zinit"], r["r_max"], r["pad"])
    w = MlOptimiserCuda(b, debug=True, **options)
    res = w.do_expectation_some_particles(batch)
    n = len(res)
    dbg = []
    for i in range(n):
        dbg.append(dict(coarse_diff2=w.debug_fetch(0, i), coarse_weight=w.debug_fetch(1, i),
                        fine_idx=w.debug_fetch(2, i), fine_diff2=w.debug_fetch(3, i),
                        fine_weight=w.debug_fetch(4, i)))
    ws = b.get_wsum()
    if int(model.get("ref_dim", 3) or 3) == 2:
        ws["prior_offset_class"] = b.get_class_offsets()
    vols = [b.get_mdl_data(k) for k in range(len(refs))]
    times = w.stage_times()
    w.close()
    b.close()
    return res, dbg, ws, vols, times


def compare(model, refs, batch, device=0, oracle_out=None, **options):
    """Error statistics of the CUDA E-step against the oracle on one batch.

    The GPU side may store only part of the coarse diff2 array (sparse
    stores of the precision form): `coarse_stored_subset` says whether its
    stored poses are among those the oracle computed, `coarse_unstored_mass`
    is the oracle's normalised weight on the poses it left out, and the
    diff2 error is taken over the stored poses.  `fine_missing_mass` /
    `fine_extra_mass` are the normalised fine weights of the oracle on poses
    the GPU did not evaluate and of the GPU on poses the oracle did not.
    `oracle_out` reuses an earlier pyoracle.run(..., debug=True) result."""
    gres, gdbg, gws, gvols, _ = run_gpu(model, refs, batch, device, **options)
    if oracle_out is None:
        oracle_out = pyoracle.run(model, refs, batch, debug=True)
    ores, odbg, ows, obpd, obpw = oracle_out
    n = len(gres)
    st = dict(coarse_diff2_rel=0.0, coarse_w_abs=0.0, sig_mismatch=0, nr_sign_diff=0,
              fine_set_mismatch=0, fine_diff2_rel=0.0, fine_w_abs=0.0, pmax_rel=0.0,
              argmax_agree=0.0, dLL_abs=0.0, sig_weight_rel=0.0, coarse_stored_subset=True,
              coarse_stored_all=True, coarse_unstored_mass=0.0, fine_missing_mass=0.0,
              fine_extra_mass=0.0, coarse_sum_rel=0.0)
    for i in range(n):
        od, gd = odbg[i]["coarse_diff2"], gdbg[i]["coarse_diff2"]
        comp = od != -999.0
        stored = np.isfinite(gd)
        st["coarse_stored_subset"] &= bool(np.all(comp[stored]))
        st["coarse_stored_all"] &= bool(np.array_equal(comp, stored))
        ow = odbg[i]["coarse_weight"] / ores["coarse_sum_weight"][i]
        st["coarse_unstored_mass"] = max(st["coarse_unstored_mass"], float(np.sum(ow[comp & ~stored])))
        st["coarse_diff2_rel"] = max(st["coarse_diff2_rel"],
                                     float(np.max(np.abs(gd[stored] - od[stored]) / np.abs(od[stored]))))
        gw = gdbg[i]["coarse_weight"] / gres["coarse_sum_weight"][i]
        st["coarse_w_abs"] = max(st["coarse_w_abs"], float(np.max(np.abs(ow - gw))))
        st["coarse_sum_rel"] = max(st["coarse_sum_rel"], abs(gres["coarse_sum_weight"][i] /
                                                             ores["coarse_sum_weight"][i] - 1.0))
        osig = odbg[i]["coarse_significant"].astype(bool)
        gsig = gdbg[i]["coarse_weight"] >= gres["coarse_significant_weight"][i]
        gsig &= gdbg[i]["coarse_weight"] > 0
        st["sig_mismatch"] = max(st["sig_mismatch"], int(np.sum(osig != gsig)))
        st["nr_sign_diff"] = max(st["nr_sign_diff"], int(abs(gres["nr_sign"][i] - ores["nr_sign"][i])))
        # fine pass: entries the oracle computed vs the GPU's list
        ofd = odbg[i]["fine_diff2"]
        ocomp = np.nonzero(ofd != -999.0)[0]
        gidx = gdbg[i]["fine_idx"]
        common, oi, gi = np.intersect1d(ocomp, gidx, return_indices=True)
        st["fine_set_mismatch"] = max(st["fine_set_mismatch"], len(ocomp) + len(gidx) - 2 * len(common))
        ofw = odbg[i]["fine_weight"] / ores["fine_sum_weight"][i]
        gfw = gdbg[i]["fine_weight"] / gres["fine_sum_weight"][i]
        st["fine_missing_mass"] = max(st["fine_missing_mass"],
                                      float(np.sum(ofw[ocomp]) - np.sum(ofw[common])))
        st["fine_extra_mass"] = max(st["fine_extra_mass"], float(np.sum(gfw) - np.sum(gfw[gi])))
        if len(common):
            o = ofd[common]
            g = gdbg[i]["fine_diff2"][gi]
            st["fine_diff2_rel"] = max(st["fine_diff2_rel"], float(np.max(np.abs(g - o) / np.abs(o))))
            ow = odbg[i]["fine_weight"][common] / ores["fine_sum_weight"][i]
            gw = gdbg[i]["fine_weight"][gi] / gres["fine_sum_weight"][i]
            st["fine_w_abs"] = max(st["fine_w_abs"], float(np.max(np.abs(ow - gw))))
        st["pmax_rel"] = max(st["pmax_rel"], abs(gres["pmax"][i] - ores["pmax"][i]) / ores["pmax"][i])
        st["argmax_agree"] += float(gres["best_ihidden_over"][i] == ores["best_ihidden_over"][i]) / n
        st["dLL_abs"] = max(st["dLL_abs"], abs(gres["dLL"][i] - ores["dLL"][i]))
        st["sig_weight_rel"] = max(st["sig_weight_rel"], abs(gres["fine_significant_weight"][i] -
                                                           ores["fine_significant_weight"][i]) /
                                   ores["fine_significant_weight"][i])
    s_o, s_g = ows["sigma2_noise"], gws["sigma2_noise"]
    nz = s_o != 0
    st["sigma2_noise_rel"] = float(np.max(np.abs(s_g[nz] - s_o[nz]) / np.abs(s_o[nz])))
    st["pdf_direction_abs"] = float(np.max(np.abs(gws["pdf_direction"] - ows["pdf_direction"])))
    st["sumw_group_rel"] = abs(gws["sumw_group"] - ows["sumw_group"]) / ows["sumw_group"]
    st["sigma2_offset_rel"] = abs(gws["sigma2_offset"] - ows["sigma2_offset"]) / max(ows["sigma2_offset"], 1e-30)
    st["LL_abs"] = abs(gws["LL"] - ows["LL"])
    if "prior_offset_class" in gws:
        o_p, g_p = ows["prior_offset_class"], gws["prior_offset_class"]
        st["prior_offset_class_rel"] = float(np.linalg.norm(g_p - o_p) / max(np.linalg.norm(o_p), 1e-30))
    bp_d = bp_w = 0.0
    for k, (gd, gw) in enumerate(gvols):
        bp_d = max(bp_d, float(np.linalg.norm(gd - obpd[k]) / np.linalg.norm(obpd[k])))
        bp_w = max(bp_w, float(np.linalg.norm(gw - obpw[k]) / np.linalg.norm(obpw[k])))
    st["bp_data_rel_l2"] = bp_d
    st["bp_weight_rel_l2"] = bp_w
    return st
