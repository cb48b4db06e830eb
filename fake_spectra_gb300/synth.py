"""Seeded synthetic particle snapshots and sightline tables.

No simulation snapshot ships with this project, so every workload is
generated: the particle fields follow closed-form relations of an overdensity
field, the sightlines follow the layouts of ``griddedspectra.py`` (regular
grid) or random placement.  Everything is generated in float64 and cast to
float32 exactly as ``Spectra._read_particle_data`` (spectra.py:550-617) does,
so the GPU path and the CPU oracle see identical float32 bits.

Units (spectra.py:593-615, 666-673): positions and smoothing lengths in
comoving kpc/h, velocities in physical km/s, temperatures in K, and the
``dens`` argument is the ion number density (cm^-3) times ``rscale`` (cm per
comoving kpc/h), so that dens x length gives a column density in cm^-2.

Interpretations made here (stated, not taken from the reference):
* "lognormal with unit mean" = exp(sigma*G - sigma^2/2); the temperature
  scatter factor uses the same unit-mean convention.
* hh = 2 (L / N^(1/3)) (delta+1)^(-1/3), the "2 x (L/32)" rule of the 32^3
  workload generalised to the mean interparticle spacing.
* delta+1 from a cloud-in-cell density of the positions is floored at 1e-3.
* Clump positions wrap periodically into the box.
"""
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

# Physical set-up shared by all workloads: z = 3, h = 0.7, flat Omega_m = 0.3.
UNIT_LENGTH_CM = 3.085678e21          # 1 kpc in cm (unitsystem.py:7)
MPC_CM = 3.085678e24


@dataclass(frozen=True)
class Transition:
    """One absorption line: wavelength (cm), damping Gamma (1/s), oscillator strength, mass (amu)."""
    name: str
    lambda_cm: float
    gamma: float
    fosc: float
    amumass: float
    species: str   # which density field feeds it: "HI" or "CIV"


LYA = Transition("lya", 1215.67e-8, 6.265e8, 0.4164, 1.00794, "HI")
LYB = Transition("lyb", 1025.72e-8, 1.897e8, 0.07912, 1.00794, "HI")
CIV = Transition("civ1548", 1548.20e-8, 2.643e8, 0.1899, 12.011, "CIV")


def cosmology(redshift=3.0, hubble=0.7, omegam=0.3):
    """(atime, rscale, velfac) as Spectra.__init__ computes them (spectra.py:210-216)."""
    atime = 1.0 / (1.0 + redshift)
    rscale = UNIT_LENGTH_CM * atime / hubble
    hz = 100.0 * hubble * np.sqrt(omegam / atime ** 3 + (1.0 - omegam))
    velfac = rscale * hz / MPC_CM
    return atime, rscale, velfac


@dataclass
class Workload:
    name: str
    box: float
    nbins: int
    velfac: float
    atime: float
    rscale: float
    kernel: int
    pos: np.ndarray          # (N, 3) float32
    vel: np.ndarray          # (N, 3) float32
    temp: np.ndarray         # (N,) float32
    hh: np.ndarray           # (N,) float32
    dens: Dict[str, np.ndarray]   # species -> (N,) float32, n_ion * rscale
    axis: np.ndarray         # (NumLos,) int32, 1-based
    cofm: np.ndarray         # (NumLos, 3) float64
    transitions: List[Transition] = field(default_factory=list)
    tautail: float = 1e-7    # spectra.py:135
    # per sightline: 1 where it was placed through a clump centre, else 0
    # (None for workloads without that placement)
    line_class: Optional[np.ndarray] = None

    @property
    def npart(self):
        return int(self.pos.shape[0])

    @property
    def nlos(self):
        return int(self.axis.shape[0])

    def call_args(self, transition, compute_tau=True, kernel=None):
        """Positional arguments of `_Particle_Interpolate` for one transition."""
        t = transition
        return (int(bool(compute_tau)), self.nbins, self.kernel if kernel is None else kernel,
                self.box, self.velfac, self.atime, t.lambda_cm, t.gamma, t.fosc, t.amumass,
                self.tautail, self.pos, self.vel, self.dens[t.species], self.temp, self.hh,
                self.axis, self.cofm)


def _lognormal_unit_mean(rng, sigma, n):
    return np.exp(sigma * rng.standard_normal(n) - 0.5 * sigma * sigma)


def cic_overdensity(pos, box, ngrid, floor=1e-3, chunk=1 << 22):
    """delta+1 at each particle from a periodic cloud-in-cell density on ngrid^3.

    Mass assignment and read-back use the same trilinear weights.  Counts are
    accumulated in float64 by np.bincount, which is order-deterministic."""
    n = pos.shape[0]
    ncell = ngrid ** 3
    grid = np.zeros(ncell, dtype=np.float64)
    scale = ngrid / box

    def corners(p):
        u = p * scale - 0.5
        i0 = np.floor(u)
        f = u - i0
        i0 = i0.astype(np.int64) % ngrid
        i1 = (i0 + 1) % ngrid
        return i0, i1, f

    for s in range(0, n, chunk):
        i0, i1, f = corners(pos[s:s + chunk].astype(np.float64))
        for cx in (0, 1):
            ix = i1[:, 0] if cx else i0[:, 0]
            wx = f[:, 0] if cx else 1.0 - f[:, 0]
            for cy in (0, 1):
                iy = i1[:, 1] if cy else i0[:, 1]
                wy = f[:, 1] if cy else 1.0 - f[:, 1]
                for cz in (0, 1):
                    iz = i1[:, 2] if cz else i0[:, 2]
                    wz = f[:, 2] if cz else 1.0 - f[:, 2]
                    grid += np.bincount((ix * ngrid + iy) * ngrid + iz, weights=wx * wy * wz,
                                        minlength=ncell)
    grid *= ncell / float(n)
    out = np.empty(n, dtype=np.float64)
    for s in range(0, n, chunk):
        i0, i1, f = corners(pos[s:s + chunk].astype(np.float64))
        acc = np.zeros(i0.shape[0], dtype=np.float64)
        for cx in (0, 1):
            ix = i1[:, 0] if cx else i0[:, 0]
            wx = f[:, 0] if cx else 1.0 - f[:, 0]
            for cy in (0, 1):
                iy = i1[:, 1] if cy else i0[:, 1]
                wy = f[:, 1] if cy else 1.0 - f[:, 1]
                for cz in (0, 1):
                    iz = i1[:, 2] if cz else i0[:, 2]
                    wz = f[:, 2] if cz else 1.0 - f[:, 2]
                    acc += grid[(ix * ngrid + iy) * ngrid + iz] * (wx * wy * wz)
        out[s:s + chunk] = acc
    return np.maximum(out, floor)


def clumpy_positions(rng, n, box, frac_clumped, nclumps, sigma, sigma_ln=None):
    """Uniform background plus isotropic Gaussian clumps (periodic).

    sigma_ln=None: every clump has width sigma; else widths are lognormal with
    median sigma and log-width sigma_ln.  Returns (positions, clump centres)."""
    centres = rng.uniform(0.0, box, size=(nclumps, 3))
    if sigma_ln is None:
        widths = np.full(nclumps, float(sigma))
    else:
        widths = sigma * np.exp(sigma_ln * rng.standard_normal(nclumps))
    ncl = int(round(frac_clumped * n))
    pos = np.empty((n, 3), dtype=np.float64)
    pos[:n - ncl] = rng.uniform(0.0, box, size=(n - ncl, 3))
    which = rng.integers(0, nclumps, size=ncl)
    pos[n - ncl:] = centres[which] + widths[which, None] * rng.standard_normal((ncl, 3))
    np.mod(pos, box, out=pos)
    perm = rng.permutation(n)
    return pos[perm], centres


def _fields(rng, delta1, n, box):
    """n_HI, T, velocities, hh from the delta+1 relations shared by all workloads."""
    nside = round(n ** (1.0 / 3.0))
    n_hi = 1e-10 * delta1 ** 1.6
    temp = 1e4 * delta1 ** 0.5 * _lognormal_unit_mean(rng, 0.3, n)
    vel = 50.0 * rng.standard_normal((n, 3))
    hh = 2.0 * (box / nside) * delta1 ** (-1.0 / 3.0)
    return n_hi, temp, vel, hh


def _finish(name, box, res, kernel, pos, vel, temp, hh, dens64, axis, cofm, transitions,
            nbins=None):
    atime, rscale, velfac = cosmology()
    if nbins is None:
        nbins = int(box * velfac / res)          # spectra.py:230
    pos32 = pos.astype(np.float32)
    # a float64 coordinate just below box may round up to box in float32
    pos32[pos32 >= np.float32(box)] = np.nextafter(np.float32(box), np.float32(0))
    dens = {k: (v * rscale).astype(np.float32) for k, v in dens64.items()}
    return Workload(name=name, box=float(box), nbins=int(nbins), velfac=float(velfac),
                    atime=float(atime), rscale=float(rscale), kernel=int(kernel),
                    pos=pos32, vel=vel.astype(np.float32), temp=temp.astype(np.float32),
                    hh=hh.astype(np.float32), dens=dens, axis=np.asarray(axis, dtype=np.int32),
                    cofm=np.asarray(cofm, dtype=np.float64), transitions=list(transitions))


def grid_sightlines(nspec, axis, box):
    """griddedspectra.py:59-88: nspec x nspec skewers along one axis."""
    a = np.arange(nspec)
    nn, mm = np.meshgrid(a, a, indexing="ij")
    nn, mm = nn.ravel(), mm.ravel()
    z = np.zeros_like(nn)
    if axis == 1:
        gid = np.stack([z, nn, mm], axis=1)
    elif axis == 2:
        gid = np.stack([nn, z, mm], axis=1)
    else:
        gid = np.stack([nn, mm, z], axis=1)
    return np.full(nspec * nspec, axis, dtype=np.int32), (box / nspec) * gid.astype(np.float64)


def random_sightlines(rng, nlos, axis, box):
    axes = np.full(nlos, axis, dtype=np.int32) if np.isscalar(axis) else np.asarray(axis)
    cofm = rng.uniform(0.0, box, size=(nlos, 3))
    return axes.astype(np.int32), cofm


def config0(seed=0):
    """32^3 uniform particles, L = 10 Mpc/h, 64 random axis-1 sightlines, 10 km/s pixels, Ly-a, cubic."""
    rng = np.random.default_rng(seed)
    n, box = 32 ** 3, 1e4
    pos = rng.uniform(0.0, box, size=(n, 3))
    delta1 = _lognormal_unit_mean(rng, 1.5, n)
    n_hi, temp, vel, hh = _fields(rng, delta1, n, box)
    axis, cofm = random_sightlines(rng, 64, 1, box)
    cofm[:, 0] = 0.0
    return _finish("config0_32cube_L1e4_64los_10kms", box, 10.0, 1, pos, vel, temp, hh,
                   {"HI": n_hi}, axis, cofm, [LYA])


def _config1_particles(rng, nside, box, ngrid, nclumps, sigma=100.0):
    n = nside ** 3
    pos, centres = clumpy_positions(rng, n, box, 0.3, nclumps, sigma)
    delta1 = cic_overdensity(pos, box, ngrid)
    n_hi, temp, vel, hh = _fields(rng, delta1, n, box)
    return pos, delta1, n_hi, temp, vel, hh, centres


def config1(seed=1, kernel=1, nside=256):
    """256^3 particles (70% uniform, 30% in 2000 clumps of 100 kpc/h), L = 60 Mpc/h,
    60x60 grid of axis-3 sightlines, 1 km/s pixels, Ly-a.  `nside` shrinks it for tests."""
    rng = np.random.default_rng(seed)
    box = 6e4
    nclumps = max(1, int(round(2000 * (nside / 256.0) ** 3)))
    pos, delta1, n_hi, temp, vel, hh, _ = _config1_particles(rng, nside, box, nside // 2, nclumps)
    axis, cofm = grid_sightlines(60, 3, box)
    return _finish("config1_%dcube_L6e4_3600los_1kms" % nside, box, 1.0, kernel, pos, vel, temp,
                   hh, {"HI": n_hi}, axis, cofm, [LYA])


def config2(seed=1, nside=256):
    """Config-1 particles with Ly-a, Ly-b and CIV 1548 (n_CIV = 10^-4.5 n_HI (delta+1)^0.3)."""
    rng = np.random.default_rng(seed)
    box = 6e4
    nclumps = max(1, int(round(2000 * (nside / 256.0) ** 3)))
    pos, delta1, n_hi, temp, vel, hh, _ = _config1_particles(rng, nside, box, nside // 2, nclumps)
    n_civ = 10 ** -4.5 * n_hi * delta1 ** 0.3
    axis, cofm = grid_sightlines(60, 3, box)
    return _finish("config2_%dcube_L6e4_3600los_1kms_3lines" % nside, box, 1.0, 1, pos, vel,
                   temp, hh, {"HI": n_hi, "CIV": n_civ}, axis, cofm, [LYA, LYB, CIV])


def config3(seed=3, nside=512, nlos=32768):
    """512^3 particles (40% in 20000 clumps, widths lognormal median 150 kpc/h, sigma_ln 0.5),
    L = 100 Mpc/h, 32768 sightlines split over axes 1/2/3 with 25% through clump centres,
    1 km/s pixels, Ly-a + Ly-b + CIV 1548.  `nside`/`nlos` shrink it for tests."""
    rng = np.random.default_rng(seed)
    box = 1e5
    n = nside ** 3
    nclumps = max(1, int(round(20000 * (nside / 512.0) ** 3)))
    pos, centres = clumpy_positions(rng, n, box, 0.4, nclumps, 150.0, sigma_ln=0.5)
    delta1 = cic_overdensity(pos, box, nside // 2)
    n_hi, temp, vel, hh = _fields(rng, delta1, n, box)
    n_civ = 10 ** -4.5 * n_hi * delta1 ** 0.3
    base = nlos // 3
    # axes 1/2/3 get 10923/10923/10922 of 32768
    counts = [base + (1 if i < nlos - 3 * base else 0) for i in range(3)]
    axis = np.concatenate([np.full(c, a + 1, dtype=np.int32) for a, c in enumerate(counts)])
    cofm = rng.uniform(0.0, box, size=(nlos, 3))
    through = rng.random(nlos) < 0.25
    pick = rng.integers(0, nclumps, size=nlos)
    cofm[through] = centres[pick[through]]
    w = _finish("config3_%dcube_L1e5_%dlos_1kms_3lines" % (nside, nlos), box, 1.0, 1, pos,
                vel, temp, hh, {"HI": n_hi, "CIV": n_civ}, axis, cofm, [LYA, LYB, CIV])
    w.line_class = through.astype(np.int8)
    return w


def config4(seed=4, nside=128, nlos=1024):
    """128^3 particles with the config-1 recipe (clump count scaled with N), L = 20 Mpc/h,
    1024 random axis-1 sightlines, 2 km/s pixels, Ly-a."""
    rng = np.random.default_rng(seed)
    box = 2e4
    nclumps = max(1, int(round(2000 * (nside / 256.0) ** 3)))
    pos, delta1, n_hi, temp, vel, hh, _ = _config1_particles(rng, nside, box, nside // 2, nclumps)
    axis, cofm = random_sightlines(rng, nlos, 1, box)
    cofm[:, 0] = 0.0
    return _finish("config4_%dcube_L2e4_%dlos_2kms" % (nside, nlos), box, 2.0, 1, pos, vel, temp,
                   hh, {"HI": n_hi}, axis, cofm, [LYA])


CONFIGS = {0: config0, 1: config1, 2: config2, 3: config3, 4: config4}


# ---------------------------------------------------------------------------
# torch generator for the large workloads (same recipes, built where the data
# is needed, in seconds).  The random streams differ from the numpy ones, so
# the two generators give different (equally valid) realisations.  The CIC
# density is accumulated in 2^-40 fixed point with integer scatter-adds, which
# makes it independent of the order of the device's atomic updates.
# ---------------------------------------------------------------------------
def _t_cic_overdensity(pos, box, ngrid, floor=1e-3, chunk=1 << 24):
    import torch
    dev = pos.device
    n = pos.shape[0]
    ncell = ngrid ** 3
    grid = torch.zeros(ncell, dtype=torch.int64, device=dev)
    scale = ngrid / box
    one = float(1 << 40)

    def corners(p):
        u = p * scale - 0.5
        i0 = torch.floor(u)
        f = u - i0
        i0 = torch.remainder(i0.to(torch.int64), ngrid)
        i1 = torch.remainder(i0 + 1, ngrid)
        return i0, i1, f

    def loop(i0, i1, f, fn):
        for cx in (0, 1):
            ix = i1[:, 0] if cx else i0[:, 0]
            wx = f[:, 0] if cx else 1.0 - f[:, 0]
            for cy in (0, 1):
                iy = i1[:, 1] if cy else i0[:, 1]
                wy = f[:, 1] if cy else 1.0 - f[:, 1]
                for cz in (0, 1):
                    iz = i1[:, 2] if cz else i0[:, 2]
                    wz = f[:, 2] if cz else 1.0 - f[:, 2]
                    fn((ix * ngrid + iy) * ngrid + iz, wx * wy * wz)

    for s in range(0, n, chunk):
        i0, i1, f = corners(pos[s:s + chunk])
        loop(i0, i1, f, lambda idx, w: grid.index_add_(0, idx, torch.round(w * one).to(torch.int64)))
    gridf = grid.to(torch.float64) * (ncell / (float(n) * one))
    out = torch.empty(n, dtype=torch.float64, device=dev)
    for s in range(0, n, chunk):
        i0, i1, f = corners(pos[s:s + chunk])
        acc = torch.zeros(i0.shape[0], dtype=torch.float64, device=dev)

        def add(idx, w, acc=acc):
            acc.add_(gridf[idx] * w)
        loop(i0, i1, f, add)
        out[s:s + chunk] = acc
    return torch.clamp(out, min=floor)


def _t_lognormal(g, sigma, n, dev):
    import torch
    return torch.exp(sigma * torch.randn(n, generator=g, device=dev, dtype=torch.float64)
                     - 0.5 * sigma * sigma)


@dataclass
class DeviceWorkload:
    """A workload whose particle arrays are float32 torch tensors (on any device)."""
    name: str
    box: float
    nbins: int
    velfac: float
    atime: float
    rscale: float
    kernel: int
    pos: object
    vel: object
    temp: object
    hh: object
    dens: Dict[str, object]
    axis: np.ndarray
    cofm: np.ndarray
    transitions: List[Transition] = field(default_factory=list)
    tautail: float = 1e-7
    line_class: Optional[np.ndarray] = None   # 1: through a clump centre (config 3)

    @property
    def npart(self):
        return int(self.pos.shape[0])

    @property
    def nlos(self):
        return int(self.axis.shape[0])

    def call_args(self, transition, compute_tau=True, kernel=None):
        t = transition
        return (int(bool(compute_tau)), self.nbins, self.kernel if kernel is None else kernel,
                self.box, self.velfac, self.atime, t.lambda_cm, t.gamma, t.fosc, t.amumass,
                self.tautail, self.pos, self.vel, self.dens[t.species], self.temp, self.hh,
                self.axis, self.cofm)

    def to_host(self):
        """The same workload with numpy arrays (for the CPU oracle)."""
        f = lambda x: x.detach().cpu().numpy()
        return Workload(name=self.name, box=self.box, nbins=self.nbins, velfac=self.velfac,
                        atime=self.atime, rscale=self.rscale, kernel=self.kernel,
                        pos=f(self.pos), vel=f(self.vel), temp=f(self.temp), hh=f(self.hh),
                        dens={k: f(v) for k, v in self.dens.items()}, axis=self.axis,
                        cofm=self.cofm, transitions=list(self.transitions),
                        tautail=self.tautail, line_class=self.line_class)


def generate_torch(config, seed=None, device="cuda", nside=None, nlos=None):
    """Config 1-4 recipes with torch random streams, arrays on `device`."""
    import torch
    spec = {
        1: dict(box=6e4, nside=256, res=1.0, frac=0.3, nclumps=2000, sigma=100.0, sigma_ln=None,
                lines=[LYA], grid=(60, 3), seed=1),
        2: dict(box=6e4, nside=256, res=1.0, frac=0.3, nclumps=2000, sigma=100.0, sigma_ln=None,
                lines=[LYA, LYB, CIV], grid=(60, 3), seed=2),
        3: dict(box=1e5, nside=512, res=1.0, frac=0.4, nclumps=20000, sigma=150.0, sigma_ln=0.5,
                lines=[LYA, LYB, CIV], nlos=32768, seed=3),
        4: dict(box=2e4, nside=128, res=2.0, frac=0.3, nclumps=250, sigma=100.0, sigma_ln=None,
                lines=[LYA], nlos=1024, seed=4),
    }[config]
    seed = spec["seed"] if seed is None else seed
    full_side = spec["nside"]
    nside = nside or full_side
    box = spec["box"]
    n = nside ** 3
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    dev = torch.device(device)
    f64 = torch.float64
    nclumps = max(1, int(round(spec["nclumps"] * (nside / full_side) ** 3)))
    centres = torch.rand(nclumps, 3, generator=g, device=dev, dtype=f64) * box
    if spec["sigma_ln"] is None:
        widths = torch.full((nclumps,), spec["sigma"], device=dev, dtype=f64)
    else:
        widths = spec["sigma"] * torch.exp(spec["sigma_ln"] * torch.randn(
            nclumps, generator=g, device=dev, dtype=f64))
    ncl = int(round(spec["frac"] * n))
    pos = torch.empty(n, 3, device=dev, dtype=f64)
    pos[:n - ncl] = torch.rand(n - ncl, 3, generator=g, device=dev, dtype=f64) * box
    which = torch.randint(0, nclumps, (ncl,), generator=g, device=dev)
    pos[n - ncl:] = centres[which] + widths[which, None] * torch.randn(
        ncl, 3, generator=g, device=dev, dtype=f64)
    del which
    pos = torch.remainder(pos, box)
    pos = pos[torch.randperm(n, generator=g, device=dev)]
    delta1 = _t_cic_overdensity(pos, box, nside // 2)
    n_hi = 1e-10 * delta1 ** 1.6
    temp = 1e4 * delta1 ** 0.5 * _t_lognormal(g, 0.3, n, dev)
    vel = 50.0 * torch.randn(n, 3, generator=g, device=dev, dtype=f64)
    hh = 2.0 * (box / nside) * delta1 ** (-1.0 / 3.0)
    dens64 = {"HI": n_hi}
    if any(t.species == "CIV" for t in spec["lines"]):
        dens64["CIV"] = 10 ** -4.5 * n_hi * delta1 ** 0.3
    del delta1
    rng = np.random.default_rng(seed)
    line_class = None
    if "grid" in spec:
        axis, cofm = grid_sightlines(spec["grid"][0], spec["grid"][1], box)
    else:
        nl = nlos or spec["nlos"]
        if config == 3:
            base = nl // 3
            counts = [base + (1 if i < nl - 3 * base else 0) for i in range(3)]
            axis = np.concatenate([np.full(c, a + 1, dtype=np.int32) for a, c in enumerate(counts)])
            cofm = rng.uniform(0.0, box, size=(nl, 3))
            through = rng.random(nl) < 0.25
            cen = centres.cpu().numpy()
            pick = rng.integers(0, nclumps, size=nl)
            cofm[through] = cen[pick[through]]
            line_class = through.astype(np.int8)
        else:
            axis, cofm = random_sightlines(rng, nl, 1, box)
            cofm[:, 0] = 0.0
    atime, rscale, velfac = cosmology()
    nbins = int(box * velfac / spec["res"])
    pos32 = pos.to(torch.float32)
    pos32[pos32 >= box] = float(np.nextafter(np.float32(box), np.float32(0)))
    del pos
    name = "config%d_%dcube_L%g_%dlos_%gkms" % (config, nside, box, len(axis), spec["res"])
    return DeviceWorkload(
        name=name, box=float(box), nbins=nbins, velfac=float(velfac), atime=float(atime),
        rscale=float(rscale), kernel=1, pos=pos32.contiguous(), vel=vel.to(torch.float32),
        temp=temp.to(torch.float32), hh=hh.to(torch.float32),
        dens={k: (v * rscale).to(torch.float32) for k, v in dens64.items()},
        axis=np.asarray(axis, dtype=np.int32), cofm=np.asarray(cofm, dtype=np.float64),
        transitions=list(spec["lines"]), line_class=line_class)
