"""Seeded synthetic E-step inputs with the shapes and statistics of the
benchmark configurations (there is no public dataset for this path).

A ground-truth volume is a sum of isotropic 3D Gaussians.  Its Fourier
transform is analytic, so both the padded Fourier reference (the
Projector::data array, low-passed to the initial resolution) and each
particle's Fourier image (central slice at a random SO(3) pose, phase-shifted,
multiplied by a CTF, plus complex white noise at the requested SNR) are
evaluated exactly, without FFTs or interpolation.  The E-step sizes
(current / coarse image sizes, pose grid) follow the reference's rules in
MlOptimiser::updateImageSizeAndResolutionPointers (src/ml_optimiser.cpp:
5684-5777).  Everything is generated in float64 with torch, on CPU or GPU.
"""
import math

import numpy as np
import torch

CONFIGS = {
    # box 64 px, 2.0 A, 2,000 particles, HEALPix order 2, psi 7.5, +/-4 px step 2
    "cfg0_box64": dict(box=64, pixel=2.0, n_particles=2000, n_blobs=300, blob_sigma=1.5,
                       blob_radius=20.0, max_shift=3.0, defocus=(10000.0, 25000.0), snr=0.05,
                       ini_high=30.0, healpix_order=2, psi_step=7.5, offset_range_px=4.0,
                       offset_step_px=2.0, diameter=100.0, classes=1),
    # box 256 px, 1.0 A, 20,000 particles, HEALPix order 3, +/-6 px step 1
    "cfg1_box256": dict(box=256, pixel=1.0, n_particles=20000, n_blobs=5000, blob_sigma=1.5,
                        blob_radius=90.0, max_shift=3.0, defocus=(8000.0, 25000.0), snr=0.03,
                        ini_high=20.0, healpix_order=3, psi_step=-1.0, offset_range_px=6.0,
                        offset_step_px=1.0, diameter=200.0, classes=1),
    # 3D classification, box 256 px, K=4: each class displaces a random 15 %
    # of a shared 4,000-Gaussian volume by 3-8 A; poses 70 % from three
    # von Mises-Fisher preferred views (kappa 5), 30 % uniform; search as box 256
    # 2D classification, box 128 px, 1.5 A, K=100: class images are projections
    # of 100 independent 500-Gaussian volumes at random poses; particles are
    # in-plane rotated, shifted (+/-4 px), CTF-modulated class images at SNR
    # 0.02; psi step 6, offsets +/-5 px step 1
    "cfg3_box128_2d": dict(box=128, pixel=1.5, n_particles=100000, n_blobs=500, blob_sigma=1.5,
                           blob_radius=30.0, max_shift=4.0, defocus=(8000.0, 30000.0), snr=0.02,
                           ini_high=20.0, healpix_order=0, psi_step=6.0, offset_range_px=5.0,
                           offset_step_px=1.0, diameter=150.0, classes=100, ref_dim=2),
    # the box-256 refinement in a late iteration: the map has reached Nyquist
    # (reference low-passed at 2 A), so the current size is the whole box
    # (256 px: 33,024 Fourier pixels per image against 1,104 in the first
    # iteration) while the coarse pass stays at 48 px; search as box 256
    "cfg1_box256_late": dict(box=256, pixel=1.0, n_particles=20000, n_blobs=5000, blob_sigma=1.5,
                             blob_radius=90.0, max_shift=3.0, defocus=(8000.0, 25000.0), snr=0.03,
                             ini_high=2.0, healpix_order=3, psi_step=-1.0, offset_range_px=6.0,
                             offset_step_px=1.0, diameter=200.0, classes=1, current_size=256,
                             coarse_size=48),
    # the late-iteration shape at box 128 (current size 128, coarse 32,
    # HEALPix order 2, psi 30 deg): a few GB on the device, for profiler
    # captures of the fine pass, weighted sums and backprojection
    "cfg1_box128_late": dict(box=128, pixel=1.0, n_particles=20000, n_blobs=2000, blob_sigma=1.5,
                             blob_radius=45.0, max_shift=3.0, defocus=(8000.0, 25000.0), snr=0.03,
                             ini_high=2.0, healpix_order=2, psi_step=30.0, offset_range_px=6.0,
                             offset_step_px=1.0, diameter=100.0, classes=1, current_size=128,
                             coarse_size=32),
    "cfg4_box256_K4": dict(box=256, pixel=1.0, n_particles=50000, n_blobs=4000, blob_sigma=1.5,
                           blob_radius=90.0, max_shift=3.0, defocus=(8000.0, 25000.0), snr=0.03,
                           ini_high=20.0, healpix_order=3, psi_step=-1.0, offset_range_px=6.0,
                           offset_step_px=1.0, diameter=200.0, classes=4,
                           class_displace=(0.15, 3.0, 8.0), views=(3, 5.0, 0.7)),
}

KV, CS, Q0 = 300.0, 2.7, 0.1


def iround(x):
    return int(x + 0.5) if x > 0 else int(x - 0.5)


def iceil(x):
    return int(x) if x == int(x) else (int(x + 1) if x > 0 else int(x))


def estep_sizes(box, pixel, ini_high, healpix_order, diameter, incr_size=10, psi_step_2d=None):
    """current_size and coarse_size of the first iteration (3D: the HEALPix
    spacing; 2D classification: the psi step is the angular sampling,
    HealpixSampling::getAngularSampling, src/healpix_sampling.cpp:1589-1598)."""
    maxres = iround(pixel * box / ini_high) + incr_size
    current = min(2 * maxres, box)
    ang = psi_step_2d if psi_step_2d else 360.0 / (6 * iround(2.0 ** healpix_order))
    coarse_res = (ang / 360.0) * math.pi * diameter / 1.2
    coarse = 2 * iceil(pixel * box / coarse_res)
    coarse = min(coarse, current)
    return current, coarse


def ctf_value(defU, defV, defAng, X, Y, kV=KV, Cs=CS, Q0=Q0, Bfac=0.0, scale=1.0, phase_shift=0.0):
    """CTF at spatial frequency (X, Y) in 1/Angstrom (CTF::getCTF, src/ctf.h:184-256)."""
    local_Cs = Cs * 1e7
    local_kV = kV * 1e3
    lam = 12.2643247 / math.sqrt(local_kV * (1.0 + local_kV * 0.978466e-6))
    K1 = math.pi / 2 * 2 * lam
    K2 = math.pi / 2 * local_Cs * lam ** 3
    K3 = math.atan(Q0 / math.sqrt(1 - Q0 * Q0))
    K4 = -Bfac / 4.0
    K5 = math.radians(phase_shift)
    a = math.radians(defAng)
    s, c = math.sin(a), math.cos(a)
    Axx = c * c * (-defU) + s * s * (-defV)
    Axy = c * s * (-defU) - s * c * (-defV)
    Ayy = s * s * (-defU) + c * c * (-defV)
    u2 = X * X + Y * Y
    gamma = K1 * (Axx * X * X + 2.0 * Axy * X * Y + Ayy * Y * Y) + K2 * u2 * u2 - K5 - K3
    ret = -torch.sin(gamma) * torch.exp(K4 * u2) * scale if torch.is_tensor(gamma) else \
        -math.sin(gamma) * math.exp(K4 * u2) * scale
    if torch.is_tensor(ret):
        small = ret.abs() < 1e-8
        ret = torch.where(small, torch.where(ret < 0, -1e-8, 1e-8) * torch.ones_like(ret), ret)
    elif abs(ret) < 1e-8:
        ret = math.copysign(1e-8, ret)
    return ret


def random_rotations(n, gen):
    """n uniform SO(3) rotation matrices (uniform unit quaternions)."""
    q = torch.randn(n, 4, generator=gen, dtype=torch.float64)
    q = q / q.norm(dim=1, keepdim=True)
    w, x, y, z = q.unbind(1)
    R = torch.stack([
        1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w),
        2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w),
        2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], dim=1)
    return R.view(n, 3, 3)


def euler_matrices(rot, tilt, psi):
    """ZYZ Euler angles (degrees, [n]) -> [n, 3, 3] matrices whose third row
    is the projection direction (Euler_angles2matrix, src/euler.cpp)."""
    a, b, g = (torch.as_tensor(v, dtype=torch.float64) * math.pi / 180.0 for v in (rot, tilt, psi))
    ca, sa, cb, sb, cg, sg = a.cos(), a.sin(), b.cos(), b.sin(), g.cos(), g.sin()
    cc, cs, sc, ss = cb * ca, cb * sa, sb * ca, sb * sa
    R = torch.stack([cg * cc - sg * sa, cg * cs + sg * ca, -cg * sb,
                     -sg * cc - cg * sa, -sg * cs + cg * ca, sg * sb,
                     sc, ss, cb], dim=-1)
    return R.view(-1, 3, 3)


def preferred_view_rotations(n, gen, views, kappa, fraction):
    """n rotations: with probability `fraction` the projection direction is
    drawn from a von Mises-Fisher distribution (concentration kappa) around
    one of the unit vectors `views` [m, 3] (chosen uniformly), else the pose
    is uniform on SO(3); psi is uniform.  vMF on the sphere by the inverse
    CDF of w = cos(angle to the mean): w = 1 + log(u + (1 - u) e^{-2 kappa}) / kappa."""
    R = random_rotations(n, gen)
    pick = torch.rand(n, generator=gen, dtype=torch.float64) < fraction
    k = int(pick.sum())
    if k == 0:
        return R
    mu = views[torch.randint(len(views), (k,), generator=gen)]
    u = torch.rand(k, generator=gen, dtype=torch.float64)
    w = 1.0 + torch.log(u + (1.0 - u) * math.exp(-2.0 * kappa)) / kappa
    phi = 2.0 * math.pi * torch.rand(k, generator=gen, dtype=torch.float64)
    # orthonormal frame (v1, v2) perpendicular to each mean direction
    helper = torch.where(mu[:, :1].abs() < 0.9, torch.tensor([1.0, 0, 0], dtype=torch.float64),
                         torch.tensor([0, 1.0, 0], dtype=torch.float64))
    v1 = torch.linalg.cross(mu, helper)
    v1 = v1 / v1.norm(dim=1, keepdim=True)
    v2 = torch.linalg.cross(mu, v1)
    st = torch.sqrt(torch.clamp(1.0 - w * w, min=0.0))[:, None]
    d = w[:, None] * mu + st * (phi.cos()[:, None] * v1 + phi.sin()[:, None] * v2)
    rot = torch.rad2deg(torch.atan2(d[:, 1], d[:, 0]))
    tilt = torch.rad2deg(torch.acos(torch.clamp(d[:, 2], -1.0, 1.0)))
    psi = 360.0 * torch.rand(k, generator=gen, dtype=torch.float64)
    R[pick] = euler_matrices(rot, tilt, psi)
    return R


class GaussianVolume:
    """Sum of isotropic Gaussians; analytic Fourier transform (cycles/pixel)."""

    def __init__(self, n_blobs, sigma, radius, gen, device="cpu"):
        c = []
        while sum(len(x) for x in c) < n_blobs:
            p = (torch.rand(4 * n_blobs, 3, generator=gen, dtype=torch.float64) * 2 - 1) * radius
            c.append(p[p.norm(dim=1) <= radius])
        self.centers = torch.cat(c)[:n_blobs].to(device)
        self.amps = (0.5 + torch.rand(n_blobs, generator=gen, dtype=torch.float64)).to(device)
        self.sigma = sigma
        self.device = device

    def displaced(self, fraction, lo, hi, gen):
        """Copy with a random `fraction` of the Gaussians moved by a random
        distance in [lo, hi] pixels along a random direction (class variants)."""
        v = GaussianVolume.__new__(GaussianVolume)
        v.sigma, v.device, v.amps = self.sigma, self.device, self.amps
        n = len(self.centers)
        m = int(round(fraction * n))
        idx = torch.randperm(n, generator=gen)[:m]
        d = torch.randn(m, 3, generator=gen, dtype=torch.float64)
        d = d / d.norm(dim=1, keepdim=True)
        dist = lo + (hi - lo) * torch.rand(m, 1, generator=gen, dtype=torch.float64)
        c = self.centers.clone().cpu()
        c[idx] += d * dist
        v.centers = c.to(self.device)
        return v

    def ft(self, k, chunk=1 << 15):
        """F(k) for k [..., 3] in cycles/pixel -> complex128 [...]."""
        shp = k.shape[:-1]
        k = k.reshape(-1, 3).to(self.device)
        out = torch.empty(k.shape[0], dtype=torch.complex128, device=self.device)
        env_c = -2.0 * math.pi ** 2 * self.sigma ** 2
        for i in range(0, k.shape[0], chunk):
            kk = k[i:i + chunk]
            ph = -2.0 * math.pi * (kk @ self.centers.T)           # [m, B]
            s = torch.polar(self.amps.expand_as(ph).contiguous(), ph).sum(1)
            out[i:i + chunk] = s * torch.exp(env_c * (kk * kk).sum(1))
        return out.reshape(shp)

    def ft_grid_separable(self, xs, ys, zs):
        """F on the tensor grid zs x ys x xs (1D frequency vectors, cycles/px)."""
        env_c = -2.0 * math.pi ** 2 * self.sigma ** 2

        def axis(v, c):  # [B, n]
            return torch.polar(torch.exp(env_c * v * v)[None, :].expand(len(c), -1).contiguous(),
                               -2.0 * math.pi * c[:, None] * v[None, :])
        gx = axis(xs.to(self.device), self.centers[:, 0])
        gy = axis(ys.to(self.device), self.centers[:, 1])
        gz = axis(zs.to(self.device), self.centers[:, 2])
        a = self.amps.to(torch.complex128)[:, None]
        m = (gy[:, :, None] * gx[:, None, :]).reshape(len(a), -1)  # [B, y*x]
        v = (gz * a).T @ m                                          # [z, y*x]
        return v.reshape(len(zs), len(ys), len(xs))


def padded_reference(vol, box, pixel, r_max, pad, lowpass_A):
    """Projector::data layout (src/projector.cpp:59-90): complex64 [z][y][x],
    logical origin x=0, y=yinit, z=zinit; zero beyond ROUND(pad*r_max)."""
    pad_size = 2 * (iround(pad * r_max) + 1) + 1
    xdim = pad_size // 2 + 1
    yinit = -(pad_size // 2)
    xs = torch.arange(xdim, dtype=torch.float64)
    ys = torch.arange(pad_size, dtype=torch.float64) + yinit
    zs = ys.clone()
    f = 1.0 / (pad * box)
    data = vol.ft_grid_separable(xs * f, ys * f, zs * f).cpu()
    r2 = xs[None, None, :] ** 2 + ys[None, :, None] ** 2 + zs[:, None, None] ** 2
    max_r2 = iround(r_max * pad) ** 2
    kA = torch.sqrt(r2) * f / pixel     # 1/Angstrom
    fc = 1.0 / lowpass_A
    w = torch.clamp((1.1 * fc - kA) / (0.2 * fc), 0.0, 1.0)
    lp = 0.5 - 0.5 * torch.cos(math.pi * w)
    data = data * lp * (r2 <= max_r2)
    return dict(data=data.to(torch.complex64).numpy(), yinit=yinit, zinit=yinit, r_max=r_max,
                pad=pad, xdim=xdim, ydim=pad_size, zdim=pad_size)


def padded_reference_2d(vol, R, box, pixel, r_max, pad, lowpass_A):
    """Padded 2D Fourier reference of the class image = projection of `vol`
    at rotation R (Projector::data of a 2D reference: complex64 [1][y][x],
    x = 0.., y from yinit; zero beyond ROUND(pad*r_max)), low-passed."""
    pad_size = 2 * (iround(pad * r_max) + 1) + 1
    xdim = pad_size // 2 + 1
    yinit = -(pad_size // 2)
    xs = torch.arange(xdim, dtype=torch.float64)
    ys = torch.arange(pad_size, dtype=torch.float64) + yinit
    X, Y = xs[None, :].expand(pad_size, xdim), ys[:, None].expand(pad_size, xdim)
    f = 1.0 / (pad * box)
    k2 = torch.stack([X * f, Y * f, torch.zeros_like(X)], -1)
    data = vol.ft(k2 @ R.to(torch.float64)).cpu()
    r2 = X ** 2 + Y ** 2
    max_r2 = iround(r_max * pad) ** 2
    kA = torch.sqrt(r2) * f / pixel
    fc = 1.0 / lowpass_A
    w = torch.clamp((1.1 * fc - kA) / (0.2 * fc), 0.0, 1.0)
    lp = 0.5 - 0.5 * torch.cos(math.pi * w)
    data = (data * lp * (r2 <= max_r2))[None]
    return dict(data=data.to(torch.complex64).numpy(), yinit=yinit, zinit=0, r_max=r_max,
                pad=pad, xdim=xdim, ydim=pad_size, zdim=1)


def inplane_matrices(psi_deg):
    """[n, 3, 3] in-plane rotations blockdiag(A(psi), 1), A = [[c, s], [-s, c]]
    (Euler_angles2matrix(0, 0, psi))."""
    a = torch.as_tensor(psi_deg, dtype=torch.float64) * math.pi / 180.0
    c, s_ = a.cos(), a.sin()
    z, o = torch.zeros_like(a), torch.ones_like(a)
    return torch.stack([c, s_, z, -s_, c, z, z, z, o], -1).view(-1, 3, 3)


def fourier_grid(size):
    """Logical (x, y) of the [size][size/2+1] FFTW half layout."""
    X = size // 2 + 1
    i = torch.arange(size, dtype=torch.float64)
    y = torch.where(i < X, i, i - size)
    x = torch.arange(X, dtype=torch.float64)
    return x[None, :].expand(size, X), y[:, None].expand(size, X)


class Dataset:
    """Seeded synthetic E-step problem for one configuration."""

    def __init__(self, cfg, seed=0, n_particles=None, device="cpu", healpix_order=None,
                 psi_step=None, offset_range_px=None, offset_step_px=None, classes=None):
        c = dict(CONFIGS[cfg]) if isinstance(cfg, str) else dict(cfg)
        if classes is not None:
            c["classes"] = classes
            c.setdefault("class_displace", (0.15, 3.0, 8.0))
        if healpix_order is not None:
            c["healpix_order"] = healpix_order
        if psi_step is not None:
            c["psi_step"] = psi_step
        if offset_range_px is not None:
            c["offset_range_px"] = offset_range_px
        if offset_step_px is not None:
            c["offset_step_px"] = offset_step_px
        self.cfg = c
        self.seed = seed
        self.device = device
        self.gen = torch.Generator().manual_seed(seed)
        self.n = int(n_particles if n_particles is not None else c["n_particles"])
        box, pix = c["box"], c["pixel"]
        self.is2d = int(c.get("ref_dim", 3)) == 2
        self.current, self.coarse = estep_sizes(box, pix, c["ini_high"], c["healpix_order"], c["diameter"],
                                                psi_step_2d=c["psi_step"] if self.is2d else None)
        # a later iteration's sizes, where the configuration gives them
        self.current = int(c.get("current_size", self.current))
        self.coarse = int(c.get("coarse_size", self.coarse))
        self.vol = GaussianVolume(c["n_blobs"], c["blob_sigma"], c["blob_radius"], self.gen, device)
        K = int(c.get("classes", 1))
        self.vols = [self.vol]
        self.class_R = None
        if self.is2d:
            # independent class volumes, each projected at its own random pose
            self.vols += [GaussianVolume(c["n_blobs"], c["blob_sigma"], c["blob_radius"], self.gen, device)
                          for _ in range(K - 1)]
            self.class_R = random_rotations(K, self.gen)
        elif K > 1:
            frac, lo, hi = c.get("class_displace", (0.15, 3.0, 8.0))
            self.vols = [self.vol.displaced(frac, lo / pix, hi / pix, self.gen) for _ in range(K)]
        self.views = None
        if c.get("views"):
            m = int(c["views"][0])
            v = torch.randn(m, 3, generator=self.gen, dtype=torch.float64)
            self.views = v / v.norm(dim=1, keepdim=True)
        self.r_max = min(self.current // 2, box // 2)
        if self.is2d:
            self.refs = [padded_reference_2d(v, self.class_R[k], box, pix, self.r_max, 2, c["ini_high"])
                         for k, v in enumerate(self.vols)]
        else:
            self.refs = [padded_reference(v, box, pix, self.r_max, 2, c["ini_high"]) for v in self.vols]
        self.ref = self.refs[0]
        self.sigma2 = None

    def model(self, precision=0):
        c = self.cfg
        box, pix = c["box"], c["pixel"]
        ndir = 1 if self.is2d else 12 * 4 ** c["healpix_order"]
        K = c["classes"]
        if self.sigma2 is None:
            self._noise_level()
        return dict(
            ori_size=box, nr_classes=K, current_size=self.current, coarse_size=self.coarse,
            padding_factor=2, healpix_order=c["healpix_order"], adaptive_oversampling=1,
            maximum_significants=-1, sigma2_len=box // 2 + 1, do_scale_correction=0,
            do_norm_correction=0, do_map=1, precision=precision, pixel_size=pix,
            psi_step=c["psi_step"], offset_range=c["offset_range_px"] * pix,
            offset_step=c["offset_step_px"] * pix, adaptive_fraction=0.999, sigma2_fudge=1.0,
            sigma2_offset=100.0, avg_norm_correction=1.0,
            sigma2_noise=np.full(box // 2 + 1, self.sigma2), pdf_class=np.full(K, 1.0 / K),
            pdf_direction=np.full(K * ndir, 1.0 / (K * ndir)), ref_dim=2 if self.is2d else 3,
            prior_offset_class=np.zeros((K, 2)) if self.is2d else None)

    def _noise_level(self):
        """sigma^2 per complex Fourier coefficient for the configured SNR:
        SNR = variance of the noise-free, CTF-modulated particle image over
        the full box (DC excluded) / noise variance, estimated on a few poses
        and defoci drawn from the configuration's distributions."""
        c = self.cfg
        box, pix = c["box"], c["pixel"]
        g = torch.Generator().manual_seed(self.seed + 7)
        nsamp = 4
        R = random_rotations(nsamp, g)
        dlo, dhi = c["defocus"]
        x, y = fourier_grid(box)
        k2 = torch.stack([x, y, torch.zeros_like(x)], -1) / box
        notdc = ~((x == 0) & (y == 0))
        p = 0.0
        for i in range(nsamp):
            dU = dlo + (dhi - dlo) * float(torch.rand(1, generator=g, dtype=torch.float64))
            dV = dlo + (dhi - dlo) * float(torch.rand(1, generator=g, dtype=torch.float64))
            dA = 180.0 * float(torch.rand(1, generator=g, dtype=torch.float64))
            f = self.vol.ft(k2 @ R[i]).cpu()
            ctf = ctf_value(dU, dV, dA, x / (box * pix), y / (box * pix))
            p += float(((f * ctf).abs() ** 2)[notdc].mean()) / nsamp
        self.signal_power = p
        self.sigma2 = p / c["snr"]

    def particles(self, start=0, count=None):
        """Particle batch [start, start+count) as host numpy arrays (E-step
        inputs at the current size) plus the true poses."""
        c = self.cfg
        if self.sigma2 is None:
            self._noise_level()
        count = self.n - start if count is None else count
        box, pix, cur = c["box"], c["pixel"], self.current
        g = torch.Generator().manual_seed(self.seed * 1000003 + start)
        K = len(self.vols)
        true_psi = None
        if self.is2d:
            # in-plane rotated class images: k3 = k2 A(psi) R_class (row vectors)
            labels = torch.randint(K, (count,), generator=g) if K > 1 else torch.zeros(count, dtype=torch.long)
            true_psi = 360.0 * torch.rand(count, generator=g, dtype=torch.float64)
            R = inplane_matrices(true_psi) @ self.class_R[labels]
        elif self.views is not None:
            _, kappa, frac = c["views"]
            R = preferred_view_rotations(count, g, self.views, float(kappa), float(frac))
        else:
            R = random_rotations(count, g)
        if not self.is2d:
            labels = torch.randint(K, (count,), generator=g) if K > 1 else torch.zeros(count, dtype=torch.long)
        shifts = (torch.rand(count, 2, generator=g, dtype=torch.float64) * 2 - 1) * c["max_shift"]
        dlo, dhi = c["defocus"]
        dU = dlo + (dhi - dlo) * torch.rand(count, generator=g, dtype=torch.float64)
        dV = dlo + (dhi - dlo) * torch.rand(count, generator=g, dtype=torch.float64)
        dA = 180.0 * torch.rand(count, generator=g, dtype=torch.float64)
        x, y = fourier_grid(cur)
        k2 = torch.stack([x, y, torch.zeros_like(x)], -1) / box
        X = cur // 2 + 1
        fimg = np.zeros((count, cur, X), np.complex64)
        fctf = np.zeros((count, cur, X), np.float32)
        s = math.sqrt(self.sigma2 / 2)
        for i in range(count):
            f = self.vols[int(labels[i])].ft(k2 @ R[i]).cpu()
            ctf = ctf_value(float(dU[i]), float(dV[i]), float(dA[i]), x / (box * pix), y / (box * pix))
            ph = torch.exp(-2j * math.pi * (x * shifts[i, 0] + y * shifts[i, 1]) / box)
            noise = torch.complex(torch.randn(cur, X, generator=g, dtype=torch.float64),
                                  torch.randn(cur, X, generator=g, dtype=torch.float64)) * s
            fimg[i] = (f * ctf * ph + noise).numpy()
            fctf[i] = ctf.numpy()
        half = box // 2 + 1
        # power beyond the current size: expected noise power per shell
        shell_cnt = np.zeros(half)
        xx, yy = fourier_grid(box)
        r = torch.round(torch.sqrt(xx ** 2 + yy ** 2)).long().numpy().ravel()
        ok = (r < half) & ~((xx.numpy().ravel() == 0) & (yy.numpy().ravel() < 0))
        np.add.at(shell_cnt, r[ok], 1)
        power = np.tile(shell_cnt * self.sigma2, (count, 1))
        beyond = shell_cnt[cur // 2 + 1:].sum()
        return dict(
            n=count, fimg=fimg, fimg_nomask=fimg.copy(), fctf=fctf, power_img=power,
            old_offset=np.zeros((count, 2)), prior=np.zeros((count, 2)),
            highres_Xi2=np.full(count, beyond * 0.5), norm_correction=np.ones(count),
            scale=np.ones(count), true_rot=R.numpy(), true_shift=shifts.numpy(),
            true_class=labels.numpy(), true_psi=None if true_psi is None else true_psi.numpy(),
            defocus=np.stack([dU.numpy(), dV.numpy(), dA.numpy()], 1))

    def particle_images(self, start=0, count=None):
        """Real-space particle images [n][box][box] (float32) of the same
        particles as particles(start, count): the full-box Fourier image
        (slice x CTF x shift + noise) transformed back with the image centre
        at box/2 and the forward-FFT normalisation 1/box^2 undone, with the
        per-particle CTF parameters and metadata of the image preparation."""
        c = self.cfg
        if self.sigma2 is None:
            self._noise_level()
        count = self.n - start if count is None else count
        box, pix = c["box"], c["pixel"]
        g = torch.Generator().manual_seed(self.seed * 1000003 + start)
        K = len(self.vols)
        if self.is2d:
            labels = torch.randint(K, (count,), generator=g) if K > 1 else torch.zeros(count, dtype=torch.long)
            psi = 360.0 * torch.rand(count, generator=g, dtype=torch.float64)
            R = inplane_matrices(psi) @ self.class_R[labels]
        else:
            R = random_rotations(count, g)
            labels = torch.randint(K, (count,), generator=g) if K > 1 else torch.zeros(count, dtype=torch.long)
        shifts = (torch.rand(count, 2, generator=g, dtype=torch.float64) * 2 - 1) * c["max_shift"]
        dlo, dhi = c["defocus"]
        dU = dlo + (dhi - dlo) * torch.rand(count, generator=g, dtype=torch.float64)
        dV = dlo + (dhi - dlo) * torch.rand(count, generator=g, dtype=torch.float64)
        dA = 180.0 * torch.rand(count, generator=g, dtype=torch.float64)
        x, y = fourier_grid(box)
        k2 = torch.stack([x, y, torch.zeros_like(x)], -1) / box
        i = torch.arange(box)[:, None]
        j = torch.arange(box // 2 + 1)[None, :]
        sign = 1.0 - 2.0 * ((i + j) % 2).to(torch.float64)
        s = math.sqrt(self.sigma2 / 2)
        imgs = np.zeros((count, box, box), np.float32)
        for n in range(count):
            f = self.vols[int(labels[n])].ft(k2 @ R[n]).cpu()
            ctf = ctf_value(float(dU[n]), float(dV[n]), float(dA[n]), x / (box * pix), y / (box * pix))
            ph = torch.exp(-2j * math.pi * (x * shifts[n, 0] + y * shifts[n, 1]) / box)
            noise = torch.complex(torch.randn(box, box // 2 + 1, generator=g, dtype=torch.float64),
                                  torch.randn(box, box // 2 + 1, generator=g, dtype=torch.float64)) * s
            F = (f * ctf * ph + noise) * sign
            imgs[n] = (torch.fft.irfft2(F, s=(box, box)) * box * box).numpy()
        ctfp = np.stack([dU.numpy(), dV.numpy(), dA.numpy(), np.zeros(count), np.ones(count), np.zeros(count)], 1)
        return dict(n=count, images=imgs, old_offset=np.zeros((count, 2)), prior=np.zeros((count, 2)),
                    norm_correction=np.ones(count), scale=np.ones(count), ctf=ctfp,
                    true_rot=R.numpy(), true_shift=shifts.numpy(), true_class=labels.numpy())

