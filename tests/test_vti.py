"""VTK ImageData loader (no vtk package): every payload form round-trips, the
Volume is built as pyvr/dataloaders/vtk_loader.py builds it, and the
reference's example files load with the properties its own tests pin
(tests/test_dataloaders/test_vtk_loader.py)."""

import os
from pathlib import Path

import numpy as np
import pytest

from pyvr_gb300 import compute_normal_volume
from pyvr_gb300.vti import load_vtk_volume, read_vti, write_vti

# the reference checkout, if present: PYVR_REFERENCE=<path to the pyvr tree>
# (the tests that read its example files skip without it)
_REFERENCE = os.environ.get("PYVR_REFERENCE")
EXAMPLES = os.path.join(_REFERENCE, "example_data") if _REFERENCE else ""


@pytest.mark.parametrize("fmt,encoding", [("ascii", "raw"), ("binary", "raw"), ("appended", "raw"),
                                          ("appended", "base64")])
@pytest.mark.parametrize("compress", [False, True])
@pytest.mark.parametrize("header_type", ["UInt32", "UInt64"])
def test_payload_forms_round_trip(tmp_path, fmt, encoding, compress, header_type):
    if fmt == "ascii" and (compress or header_type == "UInt64"):
        pytest.skip("ascii payloads have no header or compression")
    rng = np.random.default_rng(1)
    data = rng.random((5, 7, 9)).astype(np.float32)
    p = tmp_path / "v.vti"
    write_vti(p, data, spacing=(1, 2, 3), fmt=fmt, encoding=encoding, compress=compress,
              header_type=header_type, block_size=256)
    img = read_vti(p)
    assert img["dims"] == (9, 7, 5) and img["spacing"] == (1.0, 2.0, 3.0)
    el, comps = img["arrays"]["Scalars_"]
    got = img["_payload"].read(el).reshape(5, 7, 9)
    assert comps == 1 and np.array_equal(got, data)


@pytest.mark.parametrize("dtype", [np.uint8, np.int16, np.uint16, np.int32, np.float64])
def test_storage_types(tmp_path, dtype):
    data = (np.arange(4 * 3 * 2) * 7 % 250).astype(dtype).reshape(4, 3, 2)
    p = tmp_path / "t.vti"
    write_vti(p, data, compress=True)
    el, _ = read_vti(p)["arrays"]["Scalars_"]
    assert np.array_equal(read_vti(p)["_payload"].read(el).reshape(data.shape), data)


def test_volume_semantics(tmp_path):
    # anisotropic spacing and extents: bounds keep the physical aspect ratio,
    # the longest side maps to [-1, 1]; data normalised in float32
    rng = np.random.default_rng(2)
    data = (rng.random((6, 10, 20)) * 300 - 50).astype(np.float32)  # (nz, ny, nx)
    p = tmp_path / "aniso.vti"
    write_vti(p, data, spacing=(0.5, 2.0, 1.0), fmt="appended", encoding="base64", compress=True)
    v = load_vtk_volume(p)
    assert v.name == "aniso.vti(Scalars_)"
    assert v.shape == (6, 10, 20) and v.data.dtype == np.float32
    lo, hi = data.min(), data.max()
    assert np.array_equal(v.data, (data - lo) / (hi - lo))
    phys = np.array([20 * 0.5, 10 * 2.0, 6 * 1.0], np.float32)
    half = phys * np.float32(2.0 / phys.max()) / 2.0
    assert np.allclose(v.max_bounds, half) and np.allclose(v.min_bounds, -half)
    assert np.isclose(np.abs(v.max_bounds).max(), 1.0)
    assert np.array_equal(v.normals, compute_normal_volume(v.data), equal_nan=True)
    # normals left to the device layout: same data and bounds, no host normals
    w = load_vtk_volume(p, compute_normals=False)
    assert w.normals is None and np.array_equal(w.data, v.data)
    assert np.array_equal(w.min_bounds, v.min_bounds) and np.array_equal(w.max_bounds, v.max_bounds)


def test_constant_volume_and_errors(tmp_path):
    p = tmp_path / "c.vti"
    write_vti(p, np.full((3, 3, 3), 7.0, np.float32))
    assert not load_vtk_volume(str(p)).data.any()
    with pytest.raises(FileNotFoundError, match="not found"):
        load_vtk_volume(tmp_path / "missing.vti")
    with pytest.raises(ValueError, match="Available arrays.*Scalars_"):
        load_vtk_volume(p, scalars_name="InvalidName")
    p2 = tmp_path / "bad.vti"
    p2.write_text('<?xml version="1.0"?><VTKFile type="PolyData"></VTKFile>')
    with pytest.raises(ValueError):
        load_vtk_volume(p2)


@pytest.mark.skipif(not (EXAMPLES and os.path.isdir(EXAMPLES)),
                    reason="reference example data not present (set PYVR_REFERENCE)")
@pytest.mark.parametrize("name,shape", [("hydrogen", (128, 128, 128)), ("fuel", (64, 64, 64))])
def test_reference_example_files(name, shape):
    v = load_vtk_volume(Path(EXAMPLES) / f"{name}.vti")
    assert v.name == f"{name}.vti(Scalars_)" and v.shape == shape
    assert v.data.dtype == np.float32 and v.has_normals and v.normals.shape == shape + (3,)
    assert 0.0 <= v.data.min() < 0.1 and 0.9 < v.data.max() <= 1.0
    assert np.allclose(v.center, 0.0, atol=1e-6) and np.isclose(np.abs(v.max_bounds).max(), 1.0, atol=1e-6)
    assert np.allclose((v.max_bounds - v.min_bounds) / (v.max_bounds - v.min_bounds)[0], 1.0, atol=1e-6)
