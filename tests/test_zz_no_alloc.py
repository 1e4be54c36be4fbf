"""umt103_tally_noalloc: the energy edits for callers that cannot let the
library allocate device memory during a call (pool-accounted host codes,
runs with all device memory reserved up front).

The entry point works in a fixed scratch array inside the loaded library.
Checked here through the C-ABI against the allocating entry point
(umt103_tally_precision) on two calls in a row; the file is collected last so
a failure here leaves every other test already run.
"""
import numpy as np
import pytest

from umt_gb300 import capi
from umt_gb300.problems import synthetic_problem

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [capi.UMT_FP64, capi.UMT_FP32])
def test_tally_noalloc_matches_allocating_entry_point(umtlib, precision):
    torch = pytest.importorskip("torch")
    prob = synthetic_problem((3, 2, 2), 2, 2, 8, seed=21, time_dependent=True)
    m = prob.mesh
    umtlib.init(m, prob.omega, prob.weight, prob.ngr)
    umtlib.set_materials(prob.sigt, prob.sigs, prob.tau)
    umtlib.set_psi(prob.psi0, None)
    STotal = np.repeat(prob.q_ext, m.numCorner, axis=0) / (4 * np.pi)
    PsiB = np.zeros((len(prob.weight), m.nbelem, prob.ngr))
    umtlib.sweep(STotal, savePsi=True, PsiB=PsiB, precision=precision)

    ref = umtlib.tally(prob.siga, precision=precision)
    # the caller owns the device copy of the opacities
    siga_dev = torch.as_tensor(np.ascontiguousarray(prob.siga), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    first = umtlib.tally_noalloc(siga_dev.data_ptr(), precision=precision)
    # The first call on a device may make the driver load the library's device
    # image, which includes the fixed scratch array; from then on a call
    # leaves free device memory unchanged.
    free_before = torch.cuda.mem_get_info()[0]
    second = umtlib.tally_noalloc(siga_dev.data_ptr(), precision=precision)
    free_after = torch.cuda.mem_get_info()[0]
    assert free_after == free_before              # nothing was allocated on the device
    for key in ("EnergyRadiation", "PowerEscape", "PowerIncident", "PowerAbsorbed"):
        scale = max(abs(ref[key]), 1e-300)
        assert abs(first[key] - ref[key]) <= 1e-12 * scale, key
        assert second[key] == first[key], key     # fixed-order sum: bit-identical repeats
    # without opacities the absorbed power is zero and the rest unchanged
    none = umtlib.tally_noalloc(None, precision=precision)
    assert none["PowerAbsorbed"] == 0.0
    assert none["EnergyRadiation"] == first["EnergyRadiation"]


def test_tally_noalloc_with_device_memory_reserved(umtlib):
    """A caller that has already reserved (almost) all free device memory --
    the situation of a host code whose pool owns the device heap -- can still
    take the energy edits: with one tensor holding all but 64 MiB of free
    memory, the call succeeds and matches the same call made before."""
    torch = pytest.importorskip("torch")
    prob = synthetic_problem((2, 2, 2), 2, 2, 4, seed=22, time_dependent=True)
    m = prob.mesh
    umtlib.init(m, prob.omega, prob.weight, prob.ngr, flags=2 | 8)
    umtlib.set_materials(prob.sigt, prob.sigs, prob.tau)
    umtlib.set_psi(prob.psi0, None)
    STotal = np.repeat(prob.q_ext, m.numCorner, axis=0) / (4 * np.pi)
    umtlib.sweep(STotal, savePsi=True, precision=capi.UMT_FP32)
    siga_dev = torch.as_tensor(np.ascontiguousarray(prob.siga), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    before = umtlib.tally_noalloc(siga_dev.data_ptr(), precision=capi.UMT_FP32)
    free = torch.cuda.mem_get_info()[0]
    hold = torch.empty(max(free - (64 << 20), 0), dtype=torch.uint8, device="cuda")
    try:
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] < (256 << 20)        # the device is (nearly) full
        during = umtlib.tally_noalloc(siga_dev.data_ptr(), precision=capi.UMT_FP32)
    finally:
        del hold
        torch.cuda.empty_cache()
    for key in ("EnergyRadiation", "PowerEscape", "PowerIncident", "PowerAbsorbed"):
        assert during[key] == before[key], key
