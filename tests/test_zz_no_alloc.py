"""The allocation-free pair term (gbx_pair_noalloc).

It exists for callers that cannot let a library allocate device memory, such
as an engine that owns all device memory through its own pool.  These
checks call it through the C ABI, twice in a row on the same inputs (the
static scratch keeps the previous call's contents, so the second call shows
that everything that must start at zero is cleared), with and without a
pair cutoff, and compare each result with what the regular entry point
reports for the same molecule -- the total GB energy (the pair term carries
all of it, self terms included) and dE/dB -- and the pair forces with the
FP64 oracle's pair term evaluated on the same Born radii.  The tolerances
are the parity suite's.
"""
import ctypes

import numpy as np
import pytest

from openmmcustomgbintegralforce_gb300 import _lib
from openmmcustomgbintegralforce_gb300.globule import make_globule
from openmmcustomgbintegralforce_gb300.spec import GBModel
from oracle import oracle as O

pytestmark = pytest.mark.gpu

E_TOL = 2e-5
G_TOL = 1e-4
F_TOL = 1e-4


def rel_rms(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


@pytest.mark.parametrize("cutoff", [0.0, 1.0])
def test_noalloc_pair_matches_regular_entry_point_twice(cutoff):
    torch = pytest.importorskip("torch")
    g = make_globule(1000, seed=19)
    m = GBModel.charmm_gbsw(cutoff=cutoff)
    ctx = _lib.Context(m, g.n)
    ctx.set_particle_parameters(g.charge, g.radius)
    E_ref, _ = ctx.execute_host(g.positions)
    born = ctx.born_radii()
    dEdB_ref = ctx.dEdB()

    dev = torch.device("cuda:0")
    n = g.n
    stride = ((n + 31) // 32) * 32
    posq = torch.zeros((n, 4), dtype=torch.float32, device=dev)
    posq[:, :3] = torch.from_numpy(g.positions.astype(np.float32)).to(dev)
    q = torch.from_numpy(g.charge.astype(np.float32)).to(dev)
    B = torch.from_numpy(born.astype(np.float32)).to(dev)
    lib = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    results = []
    for _ in range(2):
        force = torch.zeros(3 * stride, dtype=torch.int64, device=dev)
        energy = torch.zeros(1, dtype=torch.float64, device=dev)
        dEdB = torch.zeros(n, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        st = lib.gbx_pair_noalloc(ctypes.c_void_p(posq.data_ptr()), ctypes.c_void_p(q.data_ptr()),
                                  ctypes.c_void_p(B.data_ptr()), n, m.pref, cutoff,
                                  ctypes.c_void_p(force.data_ptr()), stride, ctypes.c_void_p(energy.data_ptr()),
                                  ctypes.c_void_p(dEdB.data_ptr()), ctypes.c_void_p(stream))
        torch.cuda.synchronize()
        assert st == 0, _lib.STATUS_NAMES.get(st, st)
        results.append((float(energy.cpu()[0]), dEdB.cpu().numpy().copy(), force.cpu().numpy().copy()))
    # the pair term alone in FP64 on the same (FP32-rounded) Born radii
    ref = O.Oracle(m).pair_terms(g.positions, g.charge, born.astype(np.float32).astype(np.float64))
    for E, g_, f in results:
        assert abs(E / E_ref - 1) < E_TOL
        assert abs(E / ref["energy"] - 1) < E_TOL
        assert rel_rms(g_, dEdB_ref) < G_TOL
        fx = f.astype(np.float64) / 2.0 ** 32
        F = np.stack([fx[:n], fx[stride:stride + n], fx[2 * stride:2 * stride + n]], axis=1)
        assert rel_rms(F, ref["forces"]) < F_TOL
    # the two calls agree bit for bit: nothing leaks from the first call's scratch
    assert results[0][0] == results[1][0]
    assert np.array_equal(results[0][1], results[1][1])
    assert np.array_equal(results[0][2], results[1][2])


def test_noalloc_rejects_more_atoms_than_its_scratch():
    lib = _lib.load()
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    st = lib.gbx_pair_noalloc(dummy, dummy, dummy, 65537, -1.0, 0.0, dummy, 65537, dummy, None, None)
    assert st == 9
    assert b"static scratch" in lib.gbx_status_string(st)
