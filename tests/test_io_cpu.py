"""Checkpoint raw dumps in the reference's HDF5 object layout
(vonkarman-io/src/checkpoint.rs:25-102) and the Tier-1 Parquet schema
(vonkarman-bin/src/diagnostics_writer.rs:24-37), on the CPU."""

import numpy as np
import pytest

from vonkarman_gb300 import io as vio
from vonkarman_gb300.solver import GridSpec, ScalarDiagnostics


def fake_checkpoint(n=8):
    rng = np.random.default_rng(0)
    shp = (n, n, n // 2 + 1)
    u = [rng.standard_normal(shp) + 1j * rng.standard_normal(shp) for _ in range(3)]
    return {"u_hat": u, "time": 0.125, "step_count": 42, "dt": 1e-3, "grid": GridSpec(n), "nu": 6.25e-4}


def test_checkpoint_raw_roundtrip_is_bitwise(tmp_path):
    d = fake_checkpoint()
    p = str(tmp_path / "ck.npz")
    vio.write_checkpoint_raw(p, d, config_toml="[grid]\nn = 8\n")
    z = np.load(p)
    # the HDF5 object paths of checkpoint.rs
    for k in ("metadata/time", "metadata/step_count", "metadata/dt", "metadata/nx", "metadata/ny", "metadata/nz",
              "metadata/lx", "metadata/ly", "metadata/lz", "metadata/nu", "config/toml"):
        assert k in z.files
    for c in range(3):
        assert z[f"spectral/u_hat_re_{c}"].shape == (8, 8, 5) and z[f"spectral/u_hat_re_{c}"].dtype == np.float64
    assert z["metadata/step_count"].dtype == np.uint64
    r = vio.read_checkpoint_raw(p)
    for a, b in zip(r["u_hat"], d["u_hat"]):
        assert np.array_equal(a, b)
    assert (r["time"], r["step_count"], r["dt"], r["nu"]) == (d["time"], d["step_count"], d["dt"], d["nu"])
    assert r["grid"] == d["grid"] and r["config_toml"] == "[grid]\nn = 8\n"


def test_hdf5_converter_layout(tmp_path):
    h5py = pytest.importorskip("h5py")
    p = str(tmp_path / "ck.npz")
    vio.write_checkpoint_raw(p, fake_checkpoint(), config_toml="x")
    h = str(tmp_path / "ck.h5")
    vio.npz_to_hdf5(p, h)
    with h5py.File(h, "r") as f:
        assert f["metadata"].attrs["step_count"] == 42
        assert f["spectral/u_hat_im_2"].shape == (8, 8, 5)


def test_parquet_tier1_schema(tmp_path):
    pq = pytest.importorskip("pyarrow.parquet")
    rows = [ScalarDiagnostics(time=0.001 * i, step=i, dt=1e-3, energy=0.5 - 1e-4 * i, enstrophy=1.0, helicity=0.0,
                              superhelicity=0.0, max_vorticity=2.0, energy_dissipation_rate=-1e-3,
                              helicity_dissipation_rate=0.0, cfl_number=0.1) for i in range(1, 2501)]
    p = str(tmp_path / "diag.parquet")
    with vio.DiagnosticsWriter(p) as w:
        w.write_rows(rows)
    t = pq.read_table(p)
    assert t.column_names == list(vio.TIER1_COLUMNS)
    assert str(t.schema.field("step").type) == "uint64" and not t.schema.field("step").nullable
    assert t.num_rows == 2500
    assert t.column("step").to_pylist()[-1] == 2500
    assert abs(t.column("energy").to_pylist()[9] - (0.5 - 1e-3)) < 1e-15
