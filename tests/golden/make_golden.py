"""Generate the golden fixtures in this directory from the reference itself.

Runs only where the reference checkout exists: it compiles the unmodified
reference C++ path (oracle/build_ref.sh -> oracle/_ref/libfsref.so), feeds it
small seeded inputs and stores inputs + reference outputs as .npz files.  The
fixtures then travel with the tests to machines without the reference.

    python tests/golden/make_golden.py [reference_root [voronoi]]   (default: $FSG_REFERENCE_ROOT,
        else a "reference" directory beside this repository)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from fake_spectra_gb300 import synth  # noqa: E402


def index_fixture():
    """The 13-sightline / 9-particle table of the reference's check_index_table test
    (fake_spectra/test.cpp:164-282), restated as data."""
    lines = [(1, 4000, 4000, 4000), (1, 4000, 4000, 4000), (1, 4000, 4020, 4010),
             (1, 4000, 4000, 4010), (1, 0, 0.4, 0.1), (1, 0, 10000 - 0.4, 0.3), (1, 0, 2000, 1000),
             (3, 1000, 2000, 500), (2, 1000, 2000, 500), (1, 1000, 2000, 500),
             (3, 3000, 5000, 550), (3, 8000, 5500, 9000), (1, 6000, 5500, 9000)]
    axis = np.array([l[0] for l in lines], dtype=np.int32)
    cofm = np.array([l[1:] for l in lines], dtype=np.float64)
    pos = np.array([500, 2000, 1000, 5000, 2000.0, 1000.0, 5010.0, 2010, 990,
                    4000, 4000, 4000, 1000, 9999.9, 9999.9, 1000.5, 2000, 501,
                    7500, 7500, 7500, 4008, 4008.0, 4008.0, 2000.0, 9999, 9999.8],
                   dtype=np.float32).reshape(9, 3)
    hh = np.array([1, 1, 20, 25, 0.6, 1.5, 7, 10, 0.8], dtype=np.float32)
    return axis, cofm, pos, hh, 10000.0


def edge_fixture(seed=7):
    """Particles and sightlines crowding the periodic box edges, on all three axes,
    with duplicated sightlines and a spread of smoothing lengths."""
    rng = np.random.default_rng(seed)
    box = 1000.0
    n = 3000
    pos = rng.uniform(0, box, size=(n, 3))
    edge = rng.random((n, 3)) < 0.3
    pos[edge] = np.where(rng.random(edge.sum()) < 0.5, rng.uniform(0, 3, edge.sum()),
                         box - rng.uniform(0, 3, edge.sum()))
    hh = np.exp(rng.uniform(np.log(0.5), np.log(60), n))
    nl = 60
    axis = rng.integers(1, 4, size=nl).astype(np.int32)
    cofm = rng.uniform(0, box, size=(nl, 3))
    cofm[:10] = np.where(rng.random((10, 3)) < 0.5, rng.uniform(0, 1, (10, 3)),
                         box - rng.uniform(0, 1, (10, 3)))
    cofm[10:14] = cofm[14:18]          # duplicated sightlines
    axis[10:14] = axis[14:18]
    vel = rng.normal(0, 30, size=(n, 3))
    dens = np.exp(rng.normal(np.log(1e11), 1.0, n))
    temp = np.exp(rng.normal(np.log(1e4), 0.6, n))
    pos32 = pos.astype(np.float32)
    pos32[pos32 >= np.float32(box)] = np.float32(0.0)
    return dict(pos=pos32, vel=vel.astype(np.float32), dens=dens.astype(np.float32),
                temp=temp.astype(np.float32), hh=hh.astype(np.float32), axis=axis, cofm=cofm,
                box=box)


def subsample(w, npart, nlos, seed):
    """A small slice of a workload: `npart` random particles, `nlos` sightlines."""
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(w.npart, size=npart, replace=False))
    lidx = np.sort(rng.choice(w.nlos, size=nlos, replace=False))
    return idx, lidx


def voronoi_fixture(R, seed=21):
    """Random cells in a 1 Mpc/h box, one wrapping first cell (a particle at
    the box edge on a sightline), tau and column density with kernel 2 from the
    reference's assign_cells path (index_table.cpp:152-223)."""
    rng = np.random.default_rng(seed)
    box = 1000.0
    n = 2500
    pos = rng.uniform(0, box, size=(n, 3)).astype(np.float32)
    nl = 12
    axis = rng.integers(1, 4, nl).astype(np.int32)
    cofm = rng.uniform(0, box, size=(nl, 3))
    # sightline 0 (axis 1): a dense particle right next to it at the box edge
    axis[0] = 1
    pos[0] = [box - 0.7, cofm[0, 1] + 0.3, cofm[0, 2] - 0.2]
    vel = (30 * rng.standard_normal((n, 3))).astype(np.float32)
    dens = (rng.lognormal(0, 1, n) * 3e11).astype(np.float32)
    temp = (1e4 * rng.lognormal(0, 0.3, n)).astype(np.float32)
    hh = (60.0 * rng.lognormal(0, 0.2, n)).astype(np.float32)
    _, _, velfac = synth.cosmology()
    nbins = int(box * velfac / 0.5)
    out = dict(pos=pos, vel=vel, dens=dens, temp=temp, hh=hh, axis=axis, cofm=cofm, box=box,
               nbins=nbins, velfac=velfac)
    for t in (synth.LYA, synth.CIV):
        for ct in (0, 1):
            out["%s_%s" % ("tau" if ct else "colden", t.name)] = R.particle_interpolate(
                ct, nbins, 2, box, velfac, 0.25, t.lambda_cm, t.gamma, t.fosc, t.amumass, 1e-7,
                pos, vel, dens, temp, hh, axis, cofm)
    return out


def main(ref_root=None, only=None):
    ref_root = ref_root or oracle.reference_root()
    if not ref_root:
        raise SystemExit("reference checkout not found: set FSG_REFERENCE_ROOT")
    oracle.build_ref(ref_root)
    R = oracle.ref()
    if R is None:
        raise SystemExit("reference sources not found under %s" % ref_root)
    if only in (None, "voronoi"):
        np.savez_compressed(os.path.join(HERE, "voronoi.npz"), **voronoi_fixture(R))
        if only:
            return

    # 1. reference IndexTable fixture
    axis, cofm, pos, hh, box = index_fixture()
    off, part, dr2 = R.near_particles(pos, hh, axis, cofm, box)
    np.savez(os.path.join(HERE, "index_testcpp.npz"), axis=axis, cofm=cofm, pos=pos, hh=hh,
             box=box, off=off, part=part, dr2=dr2)

    # 2. periodic-edge fixture: pairs + tau/colden for three kernels
    e = edge_fixture()
    off, part, dr2 = R.near_particles(e["pos"], e["hh"], e["axis"], e["cofm"], e["box"])
    out = dict(e, off=off, part=part, dr2=dr2)
    _, _, velfac = synth.cosmology()
    nbins = 200
    for kernel in (0, 1, 3):
        for ct in (0, 1):
            t = synth.LYA
            res = R.particle_interpolate(ct, nbins, kernel, e["box"], velfac, 0.25, t.lambda_cm,
                                         t.gamma, t.fosc, t.amumass, 1e-7, e["pos"], e["vel"],
                                         e["dens"], e["temp"], e["hh"], e["axis"], e["cofm"])
            out["%s_k%d" % ("tau" if ct else "colden", kernel)] = res
    out["nbins"] = nbins
    out["velfac"] = velfac
    np.savez_compressed(os.path.join(HERE, "edges.npz"), **out)

    # 3. a slice of the 32^3 workload (Ly-a, cubic) with the full line set
    w = synth.config0()
    idx, lidx = subsample(w, 8192, 16, seed=11)
    args = dict(pos=w.pos[idx], vel=w.vel[idx], dens=w.dens["HI"][idx], temp=w.temp[idx],
                hh=w.hh[idx], axis=w.axis[lidx], cofm=w.cofm[lidx])
    out = dict(args, box=w.box, nbins=w.nbins, velfac=w.velfac, atime=w.atime)
    for t in (synth.LYA, synth.LYB, synth.CIV):
        for ct in (0, 1):
            res = R.particle_interpolate(ct, w.nbins, 1, w.box, w.velfac, w.atime, t.lambda_cm,
                                         t.gamma, t.fosc, t.amumass, w.tautail, args["pos"],
                                         args["vel"], args["dens"], args["temp"], args["hh"],
                                         args["axis"], args["cofm"])
            out["%s_%s" % ("tau" if ct else "colden", t.name)] = res
    off, part, dr2 = R.near_particles(args["pos"], args["hh"], args["axis"], args["cofm"], w.box)
    out.update(off=off, part=part, dr2=dr2)
    np.savez_compressed(os.path.join(HERE, "config0_slice.npz"), **out)

    # 4. Voigt profile values of the reference on a (u, a) grid
    rng = np.random.default_rng(5)
    u = np.concatenate([rng.uniform(-12, 12, 1500), rng.uniform(-400, 400, 200),
                        np.linspace(7.5, 8.5, 100), np.linspace(0, 3, 100)])
    a = np.concatenate([10 ** rng.uniform(-6, -0.5, 1700), 10 ** rng.uniform(-0.5, 0.7, 200)])
    a[:20] = 0.0
    H = np.array([R.voigt(x, y) for x, y in zip(u, a)])
    np.savez(os.path.join(HERE, "voigt.npz"), u=u, a=a, H=H)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main(*sys.argv[1:])
