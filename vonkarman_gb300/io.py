"""Checkpoint and Tier-1 series files in the reference's layouts.

* Checkpoints: the reference writes HDF5 (vonkarman-io/src/checkpoint.rs:25-102):
  group ``metadata`` with scalar attributes time, step_count, dt, nx, ny, nz,
  lx, ly, lz, nu; group ``spectral`` with datasets ``u_hat_re_c`` and
  ``u_hat_im_c`` (c = 0..2, shape (nx, ny, nz/2+1), f64, C order); group
  ``config`` with dataset ``toml`` (the config text as one f64 per byte).
  libhdf5 is not a dependency here, so ``write_checkpoint_raw`` writes the same
  objects into a NumPy ``.npz`` whose keys are the HDF5 paths
  (``metadata/time``, ``spectral/u_hat_re_0``, ``config/toml``, ...), and
  ``npz_to_hdf5`` converts such a file into the reference's HDF5 layout
  (needs h5py).  ``read_checkpoint_raw`` returns the dict that
  ``Periodic3D.from_checkpoint`` takes.
* Tier-1 time series: ``DiagnosticsWriter`` writes the Parquet schema of
  vonkarman-bin/src/diagnostics_writer.rs:24-37 (step u64, then time, dt,
  energy, enstrophy, helicity, superhelicity, max_vorticity,
  energy_dissipation_rate, helicity_dissipation_rate, cfl_number as f64;
  ZSTD) from records of ``Periodic3D.run`` (batched device readback instead
  of one read per step); it needs pyarrow and raises if it is missing.
"""

from __future__ import annotations

import numpy as np

from .solver import GridSpec

_META_F64 = ("time", "dt", "lx", "ly", "lz", "nu")
_META_U64 = ("step_count", "nx", "ny", "nz")


def write_checkpoint_raw(path: str, data: dict, config_toml: str = "") -> None:
    """Write ``Periodic3D.checkpoint_data()`` (plus the config text) as an
    ``.npz`` with the HDF5 object paths of checkpoint.rs:25-102 as keys."""
    grid: GridSpec = data["grid"]
    out = {
        "metadata/time": np.float64(data["time"]),
        "metadata/step_count": np.uint64(data["step_count"]),
        "metadata/dt": np.float64(data["dt"]),
        "metadata/nx": np.uint64(grid.n), "metadata/ny": np.uint64(grid.n), "metadata/nz": np.uint64(grid.n),
        "metadata/lx": np.float64(grid.l), "metadata/ly": np.float64(grid.l), "metadata/lz": np.float64(grid.l),
        "metadata/nu": np.float64(data["nu"]),
        "config/toml": np.frombuffer(config_toml.encode(), dtype=np.uint8).astype(np.float64),
    }
    for c, comp in enumerate(data["u_hat"]):
        comp = np.ascontiguousarray(comp, dtype=np.complex128)
        out[f"spectral/u_hat_re_{c}"] = comp.real.copy()
        out[f"spectral/u_hat_im_{c}"] = comp.imag.copy()
    with open(path, "wb") as f:
        np.savez(f, **out)


def read_checkpoint_raw(path: str) -> dict:
    """Read a file of ``write_checkpoint_raw`` into the dict of
    ``Periodic3D.checkpoint_data()`` (read_checkpoint, checkpoint.rs:107-150)."""
    z = np.load(path)
    n = int(z["metadata/nx"])
    if int(z["metadata/ny"]) != n or int(z["metadata/nz"]) != n:
        raise ValueError("only cubic grids are supported")
    l = float(z["metadata/lx"])
    u_hat = [z[f"spectral/u_hat_re_{c}"] + 1j * z[f"spectral/u_hat_im_{c}"] for c in range(3)]
    toml = bytes(np.asarray(z["config/toml"], dtype=np.float64).astype(np.uint8)).decode()
    return {"u_hat": u_hat, "time": float(z["metadata/time"]), "step_count": int(z["metadata/step_count"]),
            "dt": float(z["metadata/dt"]), "grid": GridSpec(n, l), "nu": float(z["metadata/nu"]),
            "config_toml": toml}


def npz_to_hdf5(npz_path: str, h5_path: str) -> None:
    """Convert a ``write_checkpoint_raw`` file into the reference's HDF5
    checkpoint (metadata attributes, spectral datasets, config/toml)."""
    import h5py  # documented converter dependency; not needed by anything else

    z = np.load(npz_path)
    with h5py.File(h5_path, "w") as f:
        meta = f.create_group("metadata")
        for k in _META_F64:
            meta.attrs.create(k, np.float64(z[f"metadata/{k}"]), dtype=np.float64)
        for k in _META_U64:
            meta.attrs.create(k, np.uint64(z[f"metadata/{k}"]), dtype=np.uint64)
        spec = f.create_group("spectral")
        for c in range(3):
            for part in ("re", "im"):
                spec.create_dataset(f"u_hat_{part}_{c}", data=z[f"spectral/u_hat_{part}_{c}"], dtype=np.float64)
        f.create_group("config").create_dataset("toml", data=z["config/toml"], dtype=np.float64)


TIER1_COLUMNS = ("step", "time", "dt", "energy", "enstrophy", "helicity", "superhelicity", "max_vorticity",
                 "energy_dissipation_rate", "helicity_dissipation_rate", "cfl_number")


class DiagnosticsWriter:
    """Parquet writer of Tier-1 rows with the reference's schema
    (diagnostics_writer.rs:24-37); rows are buffered and flushed every
    ``flush_interval`` rows like the reference (:46-66)."""

    def __init__(self, path: str, flush_interval: int = 1000):
        import pyarrow as pa
        import pyarrow.parquet as pq

        self._pa = pa
        self.schema = pa.schema([pa.field("step", pa.uint64(), nullable=False)] +
                                [pa.field(c, pa.float64(), nullable=False) for c in TIER1_COLUMNS[1:]])
        self._writer = pq.ParquetWriter(path, self.schema, compression="zstd")
        self._rows = []
        self.flush_interval = int(flush_interval)

    def write_row(self, diag) -> None:
        self._rows.append(diag)
        if len(self._rows) >= self.flush_interval:
            self.flush()

    def write_rows(self, diags) -> None:
        for d in diags:
            self.write_row(d)

    def flush(self) -> None:
        if not self._rows:
            return
        pa = self._pa
        cols = [pa.array([int(getattr(d, "step")) for d in self._rows], type=pa.uint64())]
        cols += [pa.array([float(getattr(d, c)) for d in self._rows], type=pa.float64()) for c in TIER1_COLUMNS[1:]]
        self._writer.write_table(pa.Table.from_arrays(cols, schema=self.schema))
        self._rows = []

    def close(self) -> None:
        self.flush()
        self._writer.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
