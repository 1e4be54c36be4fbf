"""Angular-flux checkpoint in the node layout of Teton's Conduit checkpoint.

Teton's checkpoint is a Conduit node tree that `prepForSave`
(io/ConduitCheckpoint_mod.F90:244-321) fills and `dataLoaded` (:100-225)
reads back and checks:

    num_corners                        int32
    num_phase_space_sets               int32
    corner_electron_temperature        float64[ncornr]
    phase_space_set_<k>/num_groups     int32
    phase_space_set_<k>/num_corners    int32
    phase_space_set_<k>/num_angles     int32
    phase_space_set_<k>/radiation_energy_density
                                       float64[G * ncornr * A], Psi(G, ncornr, A)
                                       in Fortran order = [A][ncornr][G] here
    geometry/Volume                    float64[ncornr]
    control_parameters/iteration/{outerTempRelTol, outerPhiRelTol, greyRelTol,
        incidentFluxRelTol, innerNLRelTol: float64;
        outerMaxIt, greyMaxIt, incidentFluxMaxIt, innerNLMaxIt: int32}

The tree is stored as a directory holding `schema.json` (for every leaf:
path, dtype, element count and byte offset) and `data.bin` (the leaves'
little-endian bytes, concatenated, each 64-byte aligned).  Conduit itself is
not a dependency; the schema keeps Conduit's leaf vocabulary (dtype names
int32/float64, number_of_elements, offset, element_bytes, endianness) so a
host code can map the leaves onto its own Conduit node.
"""
from __future__ import annotations

import json
import os

import numpy as np

DTYPES = {"int32": np.dtype("<i4"), "float64": np.dtype("<f8")}
ITERATION_CONTROLS = {
    "outerTempRelTol": "float64", "outerMaxIt": "int32", "outerPhiRelTol": "float64",
    "greyRelTol": "float64", "greyMaxIt": "int32", "incidentFluxRelTol": "float64",
    "incidentFluxMaxIt": "int32", "innerNLRelTol": "float64", "innerNLMaxIt": "int32",
}


def write_node(path: str, leaves: dict) -> None:
    """Write {'a/b/c': array-or-scalar} as schema.json + data.bin under path."""
    os.makedirs(path, exist_ok=True)
    schema, off = {}, 0
    with open(os.path.join(path, "data.bin"), "wb") as f:
        for key, value in leaves.items():
            arr = np.asarray(value)
            name = "int32" if arr.dtype.kind in "iu" else "float64"
            arr = np.ascontiguousarray(arr, dtype=DTYPES[name]).reshape(-1)
            pad = (-off) % 64
            f.write(b"\0" * pad)
            off += pad
            f.write(arr.tobytes())
            schema[key] = {"dtype": name, "number_of_elements": int(arr.size), "offset": off,
                           "element_bytes": DTYPES[name].itemsize, "endianness": "little"}
            off += arr.nbytes
    with open(os.path.join(path, "schema.json"), "w") as f:
        json.dump(schema, f, indent=1)


def read_node(path: str) -> dict:
    """Read the leaves written by write_node (scalars come back as numpy scalars)."""
    with open(os.path.join(path, "schema.json")) as f:
        schema = json.load(f)
    data = np.memmap(os.path.join(path, "data.bin"), dtype=np.uint8, mode="r")
    out = {}
    for key, s in schema.items():
        dt = DTYPES[s["dtype"]]
        arr = np.frombuffer(data, dtype=dt, count=s["number_of_elements"], offset=s["offset"]).copy()
        out[key] = arr[0] if s["number_of_elements"] == 1 else arr
    return out


def save(path: str, lib, precision: int, volume: np.ndarray, corner_temperature=None, controls=None) -> None:
    """prepForSave: the library's current angular flux (one phase-space set)."""
    Psi, _ = lib.get_psi(precision)
    A, nc, G = Psi.shape
    leaves = {
        "num_corners": np.int32(nc),
        "num_phase_space_sets": np.int32(1),
        "corner_electron_temperature": (np.zeros(nc) if corner_temperature is None else corner_temperature),
        "phase_space_set_1/num_groups": np.int32(G),
        "phase_space_set_1/num_corners": np.int32(nc),
        "phase_space_set_1/num_angles": np.int32(A),
        "phase_space_set_1/radiation_energy_density": Psi.reshape(-1),
        "geometry/Volume": volume,
    }
    ctl = dict(controls or {})
    for k, dt in ITERATION_CONTROLS.items():
        leaves["control_parameters/iteration/" + k] = (np.int32 if dt == "int32" else np.float64)(ctl.get(k, 0))
    write_node(path, leaves)


def load(path: str, lib) -> dict:
    """dataLoaded: check the sizes against the library's problem, restore Psi
    (as the saved flux of the next sweep) and return the other leaves."""
    node = read_node(path)
    checks = [("num_corners", lib.nc), ("num_phase_space_sets", 1), ("phase_space_set_1/num_groups", lib.G),
              ("phase_space_set_1/num_corners", lib.nc), ("phase_space_set_1/num_angles", lib.A)]
    for key, want in checks:
        if int(node[key]) != int(want):
            raise ValueError(f"checkpoint load error: {key} = {int(node[key])}, expected {want}")
    psi = node["phase_space_set_1/radiation_energy_density"].reshape(lib.A, lib.nc, lib.G)
    lib.set_psi(psi, None)
    return node
