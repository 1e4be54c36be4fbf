"""Angular-flux checkpoint (umt_gb300/checkpoint.py): the container round trip
on the CPU, and a restart through the library on the GPU that reproduces the
uninterrupted run bit for bit."""
import numpy as np
import pytest

from umt_gb300 import capi, checkpoint
from umt_gb300.problems import synthetic_problem


def test_node_round_trip(tmp_path):
    leaves = {"num_corners": np.int32(5), "a/b/values": np.arange(7, dtype=np.float64) / 3.0,
              "a/count": np.int32(-4), "x": np.float64(2.5), "ints": np.arange(3, dtype=np.int32)}
    checkpoint.write_node(str(tmp_path / "node"), leaves)
    back = checkpoint.read_node(str(tmp_path / "node"))
    assert set(back) == set(leaves)
    for k, v in leaves.items():
        assert np.array_equal(np.asarray(back[k]), np.asarray(v))
        assert np.asarray(back[k]).dtype.kind == np.asarray(v).dtype.kind


class _FakeLib:
    def __init__(self, A, nc, G):
        self.A, self.nc, self.G = A, nc, G
        self.psi = np.random.default_rng(0).random((A, nc, G))

    def get_psi(self, precision):
        return self.psi, None

    def set_psi(self, Psi, PsiB):
        self.psi = np.array(Psi)


def test_save_load_layout_and_size_checks(tmp_path):
    lib = _FakeLib(8, 12, 3)
    checkpoint.save(str(tmp_path / "ck"), lib, capi.UMT_FP64, volume=np.ones(12),
                    controls={"outerPhiRelTol": 1e-8, "outerMaxIt": 50})
    node = checkpoint.read_node(str(tmp_path / "ck"))
    assert int(node["phase_space_set_1/num_angles"]) == 8
    assert node["phase_space_set_1/radiation_energy_density"].shape == (8 * 12 * 3,)
    assert float(node["control_parameters/iteration/outerPhiRelTol"]) == 1e-8
    other = _FakeLib(8, 12, 3)
    checkpoint.load(str(tmp_path / "ck"), other)
    assert np.array_equal(other.psi, lib.psi)
    with pytest.raises(ValueError):
        checkpoint.load(str(tmp_path / "ck"), _FakeLib(8, 12, 4))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [capi.UMT_FP64, capi.UMT_FP32])
def test_restart_reproduces_uninterrupted_run(umtlib, tmp_path, precision):
    prob = synthetic_problem((2, 2, 1), 2, 2, 8, seed=19, time_dependent=True)
    m = prob.mesh
    STotal = np.repeat(prob.q_ext, m.numCorner, axis=0) / (4 * np.pi)

    def start():
        umtlib.init(m, prob.omega, prob.weight, prob.ngr, flags=(2 if precision == capi.UMT_FP32 else 1) | 8)
        umtlib.set_materials(prob.sigt, prob.sigs, prob.tau)

    start()
    umtlib.set_psi(prob.psi0, None)
    umtlib.sweep(STotal, savePsi=True, precision=precision)          # cycle 1
    _, _, vol = umtlib.geometry()
    checkpoint.save(str(tmp_path / "ck"), umtlib, precision, volume=vol)
    ref = umtlib.sweep(STotal, savePsi=True, precision=precision)    # cycle 2, uninterrupted
    start()                                                          # a new run restarts from the file
    node = checkpoint.load(str(tmp_path / "ck"), umtlib)
    assert np.array_equal(node["geometry/Volume"], vol)
    again = umtlib.sweep(STotal, savePsi=True, precision=precision)
    assert np.array_equal(again, ref)
