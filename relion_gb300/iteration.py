"""Refinement iterations with every step on the device: the E-step over the
particle set in batches, then the reconstruction side, then the model's
scalar update — the order MlOptimiser::iterate follows
(src/ml_optimiser.cpp: expectation :3575, maximization :4936,
maximizationOtherParameters :5090), for the path's scope: one optics group,
C1, no gradient refinement (mu = 0), a fixed current size.

Gold standard: two half-sets each with their own maps; after each iteration
the FSC of the two half-maps (getFSC) updates tau2 (updateSSNRarrays with
update_tau2_with_fsc, as auto-refine does), and the resolution at
FSC 0.143 is reported.
"""
import math

import numpy as np

from .estep import MlDeviceBundle, MlOptimiserCuda


def npix_per_shell(ori_size, data_dim=2):
    """Npix_per_shell (src/ml_optimiser.cpp:5717-5730): pixels of the FFTW
    half transform per resolution shell, the redundant half of the x = 0
    column excluded."""
    ns = ori_size // 2 + 1
    a = np.arange(ori_size)
    f = np.where(a < ns, a, a - ori_size)
    j = np.arange(ns)
    if data_dim == 3:
        kp, ip, jp = np.meshgrid(f, f, j, indexing="ij")
    else:
        kp, (ip, jp) = 0, np.meshgrid(f, j, indexing="ij")
    ires = np.floor(np.sqrt(kp * kp + ip * ip + jp * jp) + 0.5).astype(np.int64)
    keep = (ires < ns) & ~((jp == 0) & (ip < 0))
    return np.bincount(ires[keep], minlength=ns).astype(np.float64)


def maximization_other_parameters(model, wsum, npix, do_norm_correction, min_sigma2_offset=2.0,
                                  fix_sigma_noise=False, fix_sigma_offset=False, data_dim=2):
    """MlOptimiser::maximizationOtherParameters (src/ml_optimiser.cpp:5090-5300)
    with mu = 0, one optics group and one scale group: updates `model` in
    place from the weighted sums."""
    K = len(model["pdf_class"])
    sum_weight = float(np.sum(wsum["pdf_class"]))
    if sum_weight < 1e-6:  # XMIPP_EQUAL_ACCURACY
        return
    if do_norm_correction:
        model["avg_norm_correction"] = wsum["avg_norm_correction"] / sum_weight
    pdf = np.asarray(wsum["pdf_class"], np.float64) / sum_weight
    if model.get("ref_dim") == 2 and "prior_offset_class" in wsum:
        poc = np.asarray(wsum["prior_offset_class"], np.float64).reshape(K, 2) / sum_weight
        poc[np.asarray(wsum["pdf_class"]) <= 0.] = 0.
        model["prior_offset_class"] = poc.ravel()
    if pdf.sum() > 0.:
        pdf = pdf / pdf.sum()
    model["pdf_class"] = pdf
    model["pdf_direction"] = (np.asarray(wsum["pdf_direction"], np.float64) / sum_weight).ravel()
    if not fix_sigma_offset:
        div = 3. if data_dim == 3 else 2.
        model["sigma2_offset"] = max(wsum["sigma2_offset"] / (div * sum_weight), min_sigma2_offset)
    if not fix_sigma_noise:
        ws = np.asarray(wsum["sigma2_noise"], np.float64)
        if ws.sum() != 0.:
            s2 = np.array(model["sigma2_noise"], np.float64)
            for n in range(len(s2)):
                s2[n] = ws[n] / (2. * wsum["sumw_group"] * npix[n])
                if s2[n] < 1e-14 and n > 0:
                    s2[n] = s2[n - 1]
            model["sigma2_noise"] = s2
    model["LL"] = wsum["LL"]
    model["ave_Pmax"] = wsum["ave_Pmax"] / sum_weight


def update_image_sizes(model, data_vs_prior, angular_sampling_deg, particle_diameter, minres_map=5, incr_size=10,
                       split_halves=True):
    """MlOptimiser::updateCurrentResolution (src/ml_optimiser.cpp:5579-5682,
    do_map, one body, after the first iteration) and the sizes of
    updateImageSizeAndResolutionPointers (:5684-5777, incr_size, one optics
    group of the model's size): the last shell with data_vs_prior >= 1 (with
    the split-halves rule for a later rise above 1), the current size
    2 (maxres + incr_size) and the coarse size from the angular sampling.
    Updates model["current_size"], ["coarse_size"], ["current_resolution"]."""
    ori, pix = int(model["ori_size"]), float(model["pixel_size"])
    maxres = 0
    for dvp in data_vs_prior:
        ires = 1
        while ires < ori // 2 and dvp[ires] >= 1.:
            ires += 1
        ires -= 1
        if split_halves:
            ires2 = ori // 2 - 1
            while ires2 >= ires and not dvp[ires2] > 1.:
                ires2 -= 1
            if ires2 > ires + 3:
                ires = ires2
        maxres = max(maxres, ires)
    maxres = max(maxres, minres_map)
    model["current_resolution"] = maxres / (ori * pix)          # getResolution (1/Angstrom)
    cur = min(2 * (maxres + incr_size), ori)
    keepsafe = 1.2 if int(model.get("ref_dim", 3) or 3) == 3 else 1.5
    coarse_res = (angular_sampling_deg / 360.) * math.pi * particle_diameter / keepsafe
    coarse = min(2 * int(math.ceil(pix * ori / coarse_res)), cur)
    model["current_size"], model["coarse_size"] = cur, coarse


def resolution_at(fsc, ori_size, pixel_size, threshold=0.143):
    """Resolution (Angstrom) of the last shell before the FSC first drops
    below the threshold (shell 0 excluded)."""
    i = 1
    while i < len(fsc) and fsc[i] >= threshold:
        i += 1
    i = max(i - 1, 1)
    return ori_size * pixel_size / i


class HalfSet:
    """One half of the particle set with its own model and maps."""

    def __init__(self, model, maps, batches, device=0, optics=None, proposer=None):
        """batches: prepared particle batches (gbr_particle_batch fields), or,
        with `optics` (kV, Cs, Q0, particle_diameter, width_mask_edge),
        raw real-space image batches prepared on the device at each
        iteration's current size.  proposer: optional callable
        (bundle, batch) -> int32 [n][m] orientation blocks (or None) that
        restricts each batch's coarse pass (prepared batches only)."""
        self.model = dict(model)
        self.maps = [np.array(m, np.float64) for m in maps]
        self.batches = batches
        self.device = device
        self.optics = optics
        self.proposer = proposer
        if proposer is not None and optics is not None:
            raise ValueError("a proposer needs prepared particle batches")
        self.dvp = None
        K = int(model["nr_classes"])
        self.tau2 = [None] * K
        self.wsum = None
        self.last_results = []

    def expectation(self):
        """Device projectors from the maps (tau2 from their spectra, as
        MlModel::setFourierTransformMaps with update_tau2_spectra), then the
        E-step over every batch; returns the bundle holding the sums."""
        m = self.model
        b = MlDeviceBundle(m, device=self.device)
        cur = int(m["current_size"])
        for k, v in enumerate(self.maps):
            ps = b.set_fourier_transform_map(k, v, cur)
            if self.tau2[k] is None:
                self.tau2[k] = ps
        w = MlOptimiserCuda(b)
        if self.optics is not None:
            b.set_optics(**self.optics)
            self.last_results = [w.do_expectation_images(bt) for bt in self.batches]
        elif self.proposer is not None:
            self.last_results = [w.do_expectation_some_particles(bt, blocks=self.proposer(b, bt))
                                 for bt in self.batches]
            if hasattr(self.proposer, "release"):
                self.proposer.release()  # a network reading this bundle goes before the bundle
        else:
            self.last_results = [w.do_expectation_some_particles(bt) for bt in self.batches]
        w.close()
        self.wsum = b.get_wsum()
        return b

    def maximization(self, b, fsc=None, tau2_fudge=1.0, minres_map=5, gridding_iter=10):
        """Per class: symmetrise, updateSSNRarrays (with the FSC when given),
        reconstruct with the MAP term; then the scalar model update."""
        m = self.model
        self.dvp = []
        for k in range(len(self.maps)):
            b.symmetrise(k)
            s = b.update_ssnr_arrays(k, tau2_fudge, self.tau2[k], fsc, fsc is not None)
            self.tau2[k] = s["tau2"]
            self.dvp.append(s["data_vs_prior"])
            self.maps[k] = b.reconstruct(k, max_iter_preweight=gridding_iter, do_map=True, tau2=s["tau2"],
                                         tau2_fudge=tau2_fudge, normalise=self.wsum["pdf_class"][k],
                                         minres_map=minres_map)
        maximization_other_parameters(m, self.wsum, npix_per_shell(int(m["ori_size"])),
                                      bool(m.get("do_norm_correction", 0)))
        b.close()


def refine(halves, iterations, pixel_size, adapt_sizes=None):
    """Gold-standard iterations over two HalfSet objects; returns the FSC
    curve and the FSC-0.143 resolution after each iteration.  With
    adapt_sizes = dict(angular_sampling_deg=..., particle_diameter=...) the
    current and coarse sizes follow the resolution between iterations (the
    half-sets must then hold raw image batches)."""
    out = []
    fsc = None
    for _ in range(iterations):
        sizes = (int(halves[0].model["current_size"]), int(halves[0].model["coarse_size"]))
        bundles = [h.expectation() for h in halves]
        for h, b in zip(halves, bundles):
            h.maximization(b, fsc)
        b0 = MlDeviceBundle(halves[0].model, device=halves[0].device)
        fsc = b0.fsc(halves[0].maps[0], halves[1].maps[0])
        b0.close()
        if adapt_sizes is not None:
            # both halves take the sizes of the joint data_vs_prior (FSC-based after the first pass)
            for h in halves:
                update_image_sizes(h.model, halves[0].dvp + halves[1].dvp, **adapt_sizes)
        out.append(dict(fsc=fsc, resolution=resolution_at(fsc, int(halves[0].model["ori_size"]), pixel_size),
                        LL=[h.model["LL"] for h in halves], sizes=sizes))
    return out


def gaussian_map(vol, box, lowpass_px=None):
    """Real-space map of a datagen GaussianVolume on a box^3 grid (origin at
    box // 2, pixel units), scaled so that computeFourierTransformMap of it
    matches the particle images;
    optionally low-passed with a raised-cosine edge of 2 shells at radius
    lowpass_px (in Fourier pixels)."""
    c = vol.centers.detach().cpu().numpy()
    a = vol.amps.detach().cpu().numpy()
    s = float(vol.sigma)
    g = np.arange(box) - box // 2
    # the particle images' Fourier transforms are the volume's analytic
    # transform M(k) (no 1/N^2), and computeFourierTransformMap of a map
    # sampled at pixel spacing gives M / N^2: hence the N^2
    norm = (2 * math.pi * s * s) ** -1.5 * box * box
    out = np.zeros((box,) * 3)
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    for (cx, cy, cz), amp in zip(c, a):
        out += amp * norm * np.exp(-((x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2) / (2 * s * s))
    if lowpass_px is not None:
        F = np.fft.rfftn(out)
        f = np.fft.fftfreq(box) * box
        fr = np.fft.rfftfreq(box) * box
        r = np.sqrt(f[:, None, None] ** 2 + f[None, :, None] ** 2 + fr[None, None, :] ** 2)
        w = np.clip((lowpass_px + 1. - r) / 2., 0., 1.)
        w = 0.5 - 0.5 * np.cos(np.pi * w)
        out = np.fft.irfftn(F * w, s=out.shape, axes=(0, 1, 2))
    return out
