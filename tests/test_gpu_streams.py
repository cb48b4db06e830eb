"""Stream ordering: device calls made from torch run after torch's pending work
on the same stream, so inputs still being written when the call is made are
read in their final state (and the pair search's count and emit passes see
the same particles)."""
import numpy as np
import pytest

from fake_spectra_gb300 import synth

pytestmark = pytest.mark.gpu

# ~20 ms of GPU time at 2 GHz: longer than the host needs to issue the call
SLEEP_CYCLES = 40_000_000


def _inputs():
    import torch
    w = synth.config0()
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    return w, T(w.pos), T(w.vel), T(w.dens["HI"]), T(w.temp), T(w.hh)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_call_waits_for_pending_torch_work(ctx, precision):
    import torch
    from fake_spectra_gb300 import interp as I
    w, pos, vel, dens, temp, hh = _inputs()
    args = w.call_args(synth.LYA, 1)
    torch.cuda.synchronize()
    want = I.particle_interpolate_device(ctx, *args[:11], pos, vel, dens, temp, hh,
                                         args[16], args[17], precision=precision)
    torch.cuda.synchronize()
    # smoothing lengths that are still zero until a delayed copy on torch's stream
    late = torch.zeros_like(hh)
    torch.cuda.synchronize()
    torch.cuda._sleep(SLEEP_CYCLES)
    late.copy_(hh)
    got = I.particle_interpolate_device(ctx, *args[:11], pos, vel, dens, temp, late,
                                        args[16], args[17], precision=precision)
    assert torch.equal(got, want)


def test_search_waits_for_pending_torch_work(ctx, port):
    import torch
    from fake_spectra_gb300 import interp as I
    w, pos, _, _, _, hh = _inputs()
    off_o, _, _ = port.near_particles(w.pos, w.hh, w.axis, w.cofm, w.box)
    late = torch.zeros_like(hh)
    torch.cuda.synchronize()
    torch.cuda._sleep(SLEEP_CYCLES)
    late.copy_(hh)
    n = I.build_pairs(ctx, w.box, pos, late, w.axis, w.cofm)
    assert n == int(off_o[-1])
