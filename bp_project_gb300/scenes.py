"""Seeded synthetic stripmap scenes for the BP / FFBP path.

No public dataset exists for this path; the reference's own tests synthesise
range-compressed data analytically (``fast_bp/validate.py:14-25``,
``fast_bp/gpu_baseline.py:121-187``).  This module builds the benchmark
scenes the same way: a straight side-looking track, point targets and
clutter scatterers rendered as ``a * sinc((r_bin - R)/rho) * exp(-j k R)``
with the exact two-way carrier phase (``k = 4 pi fc / c``), plus circular
complex Gaussian receiver noise.  The sinc is truncated to +-``sinc_half``
range bins around each scatterer (the tail beyond 32 bins is below 1%).

Coordinates follow the reference: x cross-track (ground range), y
along-track, z height above a flat scene at z = 0.

Scenes (sizes from the benchmark definitions):

* ``c0``: 9.6 GHz, 150 MHz, fs 180 MHz, PRF 1 kHz, 100 m/s, 3 km altitude,
  4 km near slant range; 1024 pulses x 2048 bins; 512 x 512 pixels at 0.5 m;
  nine unit targets on a 3 x 3 grid; noise at 20 dB SNR.
* ``c1``: c0 geometry; 4096 x 8192; 2048 x 2048 at 0.5 m; 25 targets with
  amplitude U(1, 10) over CN(0, 0.1^2) clutter scatterers; FFBP leaves of
  16 pulses (256 leaves, 8 merge levels).
* ``c2``: 10 GHz, 300 MHz, fs 360 MHz, PRF 1.5 kHz, 150 m/s, 30 km near slant
  range (altitude not given: 3 km is used); 8192 x 16384; 4096 x 4096 at
  0.25 m; 49 targets; noise at 15 dB SNR.
* ``c3``: c0 geometry; 2048 x 4096; 1024 x 1024 at 0.5 m; 16 targets over
  clutter; trajectory errors are injected by :func:`inject_trajectory_error`.
"""
from __future__ import annotations

from dataclasses import dataclass, field, replace

import numpy as np

LIGHT_SPEED = 299792458.0


@dataclass(frozen=True)
class SceneConfig:
    name: str
    fc: float
    bandwidth: float
    fs: float
    prf: float
    speed: float
    altitude: float
    near_slant: float
    pulses: int
    samples: int
    image_side: int
    pixel_spacing: float
    n_targets: int
    target_amplitude: tuple = (1.0, 1.0)
    target_grid: bool = False
    clutter_scatterers: int = 0
    clutter_sigma: float = 0.0
    snr_db: float | None = None
    leaf_size: int = 16
    range_spacing: float = 0.25
    angular_oversample: float = 2.5
    seed: int = 2026
    sinc_half: int = 32

    # Derived geometry ------------------------------------------------------
    @property
    def data_dr(self) -> float:
        return LIGHT_SPEED / (2.0 * self.fs)

    @property
    def k(self) -> float:
        return 4.0 * np.pi * self.fc / LIGHT_SPEED

    @property
    def wavelength(self) -> float:
        return LIGHT_SPEED / self.fc

    @property
    def resolution(self) -> float:
        return LIGHT_SPEED / (2.0 * self.bandwidth)

    @property
    def near_ground(self) -> float:
        return float(np.sqrt(self.near_slant**2 - self.altitude**2))

    @property
    def pulse_spacing(self) -> float:
        return self.speed / self.prf

    @property
    def range_start(self) -> float:
        # A margin of 128 bins before the nearest scene point.
        return self.near_slant - 128.0 * self.data_dr

    @property
    def scene_centre(self) -> tuple:
        half = 0.5 * self.image_side * self.pixel_spacing
        return (self.near_ground + half, 0.0)

    @property
    def n_pixels(self) -> int:
        return self.image_side * self.image_side


CONFIGS = {
    "c0": SceneConfig("c0", 9.6e9, 150e6, 180e6, 1e3, 100.0, 3000.0, 4000.0, 1024, 2048, 512, 0.5,
                      9, target_grid=True, snr_db=20.0, leaf_size=64),
    "c1": SceneConfig("c1", 9.6e9, 150e6, 180e6, 1e3, 100.0, 3000.0, 4000.0, 4096, 8192, 2048, 0.5,
                      25, target_amplitude=(1.0, 10.0), clutter_scatterers=2048, clutter_sigma=0.1,
                      leaf_size=16),
    "c2": SceneConfig("c2", 10e9, 300e6, 360e6, 1.5e3, 150.0, 3000.0, 30000.0, 8192, 16384, 4096, 0.25,
                      49, snr_db=15.0, leaf_size=16),
    "c3": SceneConfig("c3", 9.6e9, 150e6, 180e6, 1e3, 100.0, 3000.0, 4000.0, 2048, 4096, 1024, 0.5,
                      16, target_amplitude=(1.0, 10.0), clutter_scatterers=1024, clutter_sigma=0.1,
                      leaf_size=16),
}


def batch_configs(count: int = 64, seed: int = 4096, pulse_choices=None, side_choices=(256, 512, 1024, 2048),
                  near_range=(3.5e3, 8.0e3)):
    """The uneven multi-scene workload: ``count`` scenes with the 1024-pulse scene's radar
    (9.6 GHz, 150 MHz, 180 MHz sampling, 1 kHz PRF, 100 m/s, 3 km altitude) and

    * pulses uniform over {512, 1024, ..., 8192},
    * image side uniform over {256, 512, 1024, 2048} at 0.5 m,
    * near slant range uniform in ``near_range`` (the lower end is 3.5 km, not 3 km:
      at 3 km altitude a 3 km slant range is the nadir point, where ground range is 0),
    * 4..16 seeded point targets (amplitude 1..10) over 256 clutter scatterers, no noise,
    * half direct BP, half FFBP (leaves of 16 pulses), in seeded random order.

    Range bins per scene cover the image from every pulse (rounded up to 256).
    Returns a list of (SceneConfig, kind) with kind "direct" or "ffbp"."""
    rng = np.random.default_rng(seed)
    base = CONFIGS["c0"]
    pulse_choices = np.arange(512, 8193, 512) if pulse_choices is None else np.asarray(pulse_choices)
    kinds = rng.permutation(np.array(["direct", "ffbp"] * ((count + 1) // 2))[:count])
    out = []
    for i in range(count):
        pulses = int(rng.choice(pulse_choices))
        side = int(rng.choice(side_choices))
        near = float(rng.uniform(*near_range))
        cfg = replace(base, name=f"batch{i}", pulses=pulses, image_side=side, near_slant=near,
                      n_targets=int(rng.integers(4, 17)), target_grid=False, target_amplitude=(1.0, 10.0),
                      clutter_scatterers=256, clutter_sigma=0.1, snr_db=None, leaf_size=16,
                      seed=int(rng.integers(1 << 30)))
        half_ap = 0.5 * pulses * cfg.pulse_spacing
        far_ground = cfg.near_ground + side * cfg.pixel_spacing
        far = float(np.sqrt(far_ground**2 + (0.5 * side * cfg.pixel_spacing + half_ap) ** 2 + cfg.altitude**2))
        samples = int(np.ceil(((far - cfg.range_start) / cfg.data_dr + 160) / 256.0) * 256)
        out.append((replace(cfg, samples=samples), str(kinds[i])))
    return out


def scaled(config: SceneConfig, pulses: int | None = None, samples: int | None = None,
           image_side: int | None = None, **kw) -> SceneConfig:
    """A smaller scene with the same geometry (used for parity checks)."""
    changes = dict(kw)
    if pulses is not None:
        changes["pulses"] = int(pulses)
    if samples is not None:
        changes["samples"] = int(samples)
    if image_side is not None:
        changes["image_side"] = int(image_side)
    return replace(config, **changes)


@dataclass
class Lattice:
    """Pixel (i, j) sits at ``origin + i*step_row + j*step_col``; image is [rows, cols]."""
    origin: np.ndarray
    step_row: np.ndarray
    step_col: np.ndarray
    rows: int
    cols: int

    def points(self) -> np.ndarray:
        i = np.arange(self.rows, dtype=np.float64)[:, None, None]
        j = np.arange(self.cols, dtype=np.float64)[None, :, None]
        pts = self.origin[None, None, :] + i * self.step_row[None, None, :] + j * self.step_col[None, None, :]
        return np.ascontiguousarray(pts.reshape(-1, 3))

    def take(self, flat_index) -> np.ndarray:
        flat_index = np.asarray(flat_index)
        i = (flat_index // self.cols).astype(np.float64)[:, None]
        j = (flat_index % self.cols).astype(np.float64)[:, None]
        return self.origin[None, :] + i * self.step_row[None, :] + j * self.step_col[None, :]


@dataclass
class Scene:
    config: SceneConfig
    data: np.ndarray          # complex64 [pulses, samples]
    position: np.ndarray      # float64 [pulses, 3]
    weight: np.ndarray        # float64 [pulses]
    phase: np.ndarray         # float64 [pulses]
    targets: np.ndarray       # float64 [T, 3]
    amplitudes: np.ndarray    # complex128 [T]
    lattice: Lattice
    extent: tuple             # (rmin, rmax, umin, umax) about the full-aperture mean origin
    side: int = 1
    extra: dict = field(default_factory=dict)

    @property
    def range_start(self) -> float:
        return self.config.range_start

    @property
    def data_dr(self) -> float:
        return self.config.data_dr

    @property
    def k(self) -> float:
        return self.config.k

    @property
    def fc(self) -> float:
        return self.config.fc


def trajectory(config: SceneConfig) -> np.ndarray:
    """Straight track along y at x = 0, z = altitude, centred on y = 0."""
    n = np.arange(config.pulses, dtype=np.float64)
    y = (n - 0.5 * (config.pulses - 1)) * config.pulse_spacing
    return np.column_stack([np.zeros_like(y), y, np.full_like(y, config.altitude)])


def lattice(config: SceneConfig) -> Lattice:
    """Ground image: rows run in x (cross-track), columns in y (along-track)."""
    n, s = config.image_side, config.pixel_spacing
    xc, yc = config.scene_centre
    origin = np.array([xc - 0.5 * (n - 1) * s, yc - 0.5 * (n - 1) * s, 0.0])
    return Lattice(origin, np.array([s, 0.0, 0.0]), np.array([0.0, s, 0.0]), n, n)


def polar_extent(config: SceneConfig, position: np.ndarray, margin: float = 2.0) -> tuple:
    """Slant-range / sin(angle) sector about the mean track point covering the ground image."""
    lat = lattice(config)
    o = position.mean(axis=0)
    corners_i = np.array([0, lat.rows - 1])
    corners_j = np.array([0, lat.cols - 1])
    xs = lat.origin[0] + corners_i * lat.step_row[0]
    ys = lat.origin[1] + corners_j * lat.step_col[1]
    xx, yy = np.meshgrid(xs, ys, indexing="ij")
    dx, dy = xx - o[0], yy - o[1]
    g = np.sqrt(dx * dx + dy * dy)
    r = np.sqrt(g * g + o[2] ** 2)
    # Nearest slant range is on the near edge at y = o_y (inside the image span).
    gmin = float(np.abs(xs - o[0]).min())
    rmin = float(np.sqrt(gmin**2 + o[2] ** 2))
    u = dy / g
    return (rmin - margin, float(r.max()) + margin, float(u.min()) - 1e-3, float(u.max()) + 1e-3)


def _targets(config: SceneConfig, rng: np.random.Generator):
    n, s = config.image_side, config.pixel_spacing
    xc, yc = config.scene_centre
    half = 0.5 * n * s
    if config.target_grid:
        side = int(round(np.sqrt(config.n_targets)))
        offs = (np.arange(side) - 0.5 * (side - 1)) * (half / 2.0)
        xx, yy = np.meshgrid(offs, offs, indexing="ij")
        # Off-grid by a fraction of a pixel so no target sits exactly on a pixel centre.
        pts = np.column_stack([xc + xx.ravel() + 0.13 * s, yc + yy.ravel() + 0.29 * s,
                               np.zeros(xx.size)])
        amp = np.ones(len(pts), np.complex128)
    else:
        pts = np.column_stack([xc + rng.uniform(-0.8, 0.8, config.n_targets) * half,
                               yc + rng.uniform(-0.8, 0.8, config.n_targets) * half,
                               np.zeros(config.n_targets)])
        lo, hi = config.target_amplitude
        amp = rng.uniform(lo, hi, config.n_targets) * np.exp(2j * np.pi * rng.uniform(size=config.n_targets))
    return pts, amp


def render(config: SceneConfig, position: np.ndarray, scatterers: np.ndarray, amplitudes: np.ndarray,
           range_start: float | None = None, device: str = "cpu") -> np.ndarray:
    """Range-compressed complex64 data of point scatterers (exact two-way carrier phase).

    Evaluated in float64 with torch on ``device`` ("cpu" or a CUDA device), in
    chunks of scatterers; returns a host complex64 array [pulses, samples].
    """
    import torch

    r0 = config.range_start if range_start is None else range_start
    dr, rho, k, h = config.data_dr, config.resolution, config.k, config.sinc_half
    dev = torch.device(device)
    f64 = torch.float64
    pos = torch.as_tensor(np.ascontiguousarray(position, np.float64), device=dev)
    pts = torch.as_tensor(np.ascontiguousarray(scatterers, np.float64).reshape(-1, 3), device=dev)
    amp = np.asarray(amplitudes, np.complex128).reshape(-1)
    amp_re = torch.as_tensor(amp.real.copy(), device=dev)
    amp_im = torch.as_tensor(amp.imag.copy(), device=dev)
    p, s = config.pulses, config.samples
    # One spare column per row receives the taps that fall outside the range window.
    acc_re = torch.zeros(p * (s + 1), dtype=f64, device=dev)
    acc_im = torch.zeros_like(acc_re)
    offsets = torch.arange(-h, h + 1, device=dev, dtype=torch.int64)
    row_base = (torch.arange(p, device=dev, dtype=torch.int64) * (s + 1))[None, :, None]
    chunk = max(1, int(2**24 // (p * offsets.numel())))
    for c in range(0, pts.shape[0], chunk):
        t = pts[c:c + chunk]                                                  # [S, 3]
        rng_ = torch.sqrt(((pos[None, :, :] - t[:, None, :]) ** 2).sum(-1))   # [S, P]
        bins = torch.floor((rng_ - r0) / dr).to(torch.int64)[:, :, None] + offsets[None, None, :]
        rb = r0 + bins.to(f64) * dr
        env = torch.sinc((rb - rng_[:, :, None]) / rho)                        # [S, P, W]
        ph = -k * rng_
        cr, ci = torch.cos(ph), torch.sin(ph)
        ar, ai = amp_re[c:c + chunk, None], amp_im[c:c + chunk, None]
        pr = (ar * cr - ai * ci)[:, :, None] * env
        pi = (ar * ci + ai * cr)[:, :, None] * env
        bins = torch.where((bins >= 0) & (bins < s), bins, torch.full_like(bins, s))
        flat = (row_base + bins).reshape(-1)
        acc_re.index_add_(0, flat, pr.reshape(-1))
        acc_im.index_add_(0, flat, pi.reshape(-1))
    out = torch.complex(acc_re, acc_im).reshape(p, s + 1)[:, :s].to(torch.complex64)
    return out.cpu().numpy()


def synthesize(config: SceneConfig, with_noise: bool = True, device: str = "cpu") -> Scene:
    """Build the seeded scene: trajectory, targets, clutter, noise, lattice and polar extent.

    ``device`` selects where the scatterer sum is evaluated (see :func:`render`).
    """
    rng = np.random.default_rng(config.seed)
    position = trajectory(config)
    targets, amps = _targets(config, rng)
    scat, samp = targets, amps
    if config.clutter_scatterers:
        n, s = config.image_side, config.pixel_spacing
        xc, yc = config.scene_centre
        half = 0.5 * n * s
        cl = np.column_stack([xc + rng.uniform(-1, 1, config.clutter_scatterers) * half,
                              yc + rng.uniform(-1, 1, config.clutter_scatterers) * half,
                              np.zeros(config.clutter_scatterers)])
        ca = config.clutter_sigma * (rng.standard_normal(config.clutter_scatterers)
                                     + 1j * rng.standard_normal(config.clutter_scatterers)) / np.sqrt(2.0)
        scat = np.vstack([targets, cl])
        samp = np.concatenate([amps, ca])
    data = render(config, position, scat, samp, device=device)
    if with_noise and config.snr_db is not None:
        sigma = np.sqrt(10.0 ** (-config.snr_db / 10.0) / 2.0)
        noise = rng.standard_normal(data.shape, dtype=np.float32) + 1j * rng.standard_normal(data.shape, dtype=np.float32)
        data += (sigma * noise).astype(np.complex64)
    weight = np.ones(config.pulses)
    phase = np.zeros(config.pulses)
    return Scene(config, data, position, weight, phase, targets, amps, lattice(config),
                 polar_extent(config, position))


def inject_trajectory_error(scene: Scene, los_amplitude: float = 0.02, walk_sigma: float = 1e-3,
                            quadratic_phase: float = 3 * np.pi, seed: int = 7):
    """Perturbed navigation for the autofocus scene.

    Returns (position_error [P,3], phase_error [P]): a line-of-sight sinusoid of
    ``los_amplitude`` metres with a period of one third of the aperture, a
    random walk with ``walk_sigma`` metres per pulse (detrended), and a
    quadratic phase error of ``quadratic_phase`` radians at the aperture edge.
    The data were formed on the true track; imaging uses ``position + error``.
    """
    cfg = scene.config
    rng = np.random.default_rng(seed)
    p = cfg.pulses
    t = np.arange(p) / p
    centre = np.array([*cfg.scene_centre, 0.0])
    los = centre - scene.position.mean(axis=0)
    los /= np.linalg.norm(los)
    sinus = los_amplitude * np.sin(2 * np.pi * 3 * t)
    walk = np.cumsum(rng.normal(0.0, walk_sigma, size=(p, 3)), axis=0)
    walk -= np.linspace(walk[0], walk[-1], p)
    err = sinus[:, None] * los[None, :] + walk
    x = 2 * t - 1
    phase_err = quadratic_phase * x * x
    return err, phase_err
