"""Diagnostics: ``scalars.txt`` in the reference's text layout, and field dumps.

DiagScalar mirrors the reference's DiagnosticScalar (src/Diagnostic/
DiagnosticScalar.cpp): the same scalar names in the same order, the same
two-part header and the same fixed-width scientific columns
(DiagnosticScalar.cpp:350-400), so readers of the reference's scalars.txt
(happi's Scalar) read this file unchanged.  The energy balance follows
SmileiMPI::computeGlobalDiags (src/SmileiMPI/SmileiMPI.cpp:2343-2425):
Utot = Ukin + Uelm + Urad, Uexp = Utot at step 0 plus boundary and
moving-window terms (all zero on a periodic grid), Ubal = Utot - Uexp,
Ubal_norm = Ubal / Utot.

Sums over particles and fields are FP64 reductions on the device.  Field
minima and maxima with their cell (ExMin, ExMinCell, ...) are taken on the
host from the downloaded field, at diagnostic steps only.  The cell index is
i * N1 * N2 + j * N2 + k over the N physical points per dimension.
Energies count the N physical points of the periodic grid, the convention of
a run with several patches per dimension.
"""
from __future__ import annotations

import numpy as np

GENERAL = ["Ubal_norm", "Ubal", "Utot", "Uexp", "Ukin", "Urad", "UmBWpairs", "Uelm", "Ukin_bnd", "Ukin_out_mvw",
           "Ukin_inj_mvw", "Ukin_new", "Uelm_bnd", "Uelm_out_mvw", "Uelm_inj_mvw"]
SPECIES = ["Dens_", "Ntot_", "Zavg_", "Ukin_", "Urad_"]
ENERGY_FIELDS = ["Ex", "Ey", "Ez", "Bx_m", "By_m", "Bz_m"]
MINMAX_FIELDS = ["Ex", "Ey", "Ez", "Bx_m", "By_m", "Bz_m", "Jx", "Jy", "Jz", "Rho"]
OVERSIZE = 2


def column_width(name: str, precision: int) -> int:
    """Width of a scalar's column (DiagnosticScalar::calculateWidth)."""
    return 2 + max(len(name), precision + 8)


def _sci(v: float, precision: int, width: int) -> str:
    return f"{v:>{width}.{precision}e}"


class DiagScalar:
    """Writes one row of scalars every ``every`` steps; ``vars`` restricts the columns like the namelist's."""

    def __init__(self, sim, path="scalars.txt", every=1, precision=10, vars=None):
        self.sim = sim
        self.path = path
        self.every = int(every)
        self.precision = int(precision)
        self.vars = list(vars) if vars else None
        self.energy_time_zero = 0.0
        self.latest = -1
        self._header_written = False

    # ---- columns ------------------------------------------------------------
    def _allowed(self, name: str) -> bool:
        return self.vars is None or name in self.vars

    def columns(self):
        """[(name, second name or None)] in the reference's order, filtered by ``vars``."""
        cols = [(n, None) for n in GENERAL]
        for sp in self.sim.species:
            cols += [(p + sp["name"], None) for p in SPECIES]
        cols += [("Uelm_" + f, None) for f in ENERGY_FIELDS]
        for f in MINMAX_FIELDS:
            cols += [(f + "Min", f + "MinCell"), (f + "Max", f + "MaxCell")]
        axes = "XYZ"[: self.sim.ndim]
        for side in ("min", "max"):
            for a in axes:
                cols += [(f"Poy{a}{side}", None), (f"Poy{a}{side}Inst", None)]
        return [c for c in cols if self._allowed(c[0])]

    # ---- values -----------------------------------------------------------------
    def _interior(self, a: np.ndarray) -> np.ndarray:
        sl = tuple(slice(OVERSIZE, OVERSIZE + n) for n in self.sim.n_cells)
        return a[sl]

    def values(self, itime: int) -> dict:
        sim = self.sim
        v = {n: 0.0 for n in GENERAL}
        ukin = 0.0
        for i, sp in enumerate(sim.species):
            dens, ntot, qdens, uk = sim.species_scalars(i)
            name = sp["name"]
            v["Dens_" + name] = dens
            v["Ntot_" + name] = ntot
            v["Zavg_" + name] = qdens / dens if dens != 0.0 else 0.0
            v["Ukin_" + name] = uk
            v["Urad_" + name] = 0.0
            ukin += uk
        fe = sim.field_energies()
        for f, e in zip(ENERGY_FIELDS, fe):
            v["Uelm_" + f] = float(e)
        v["Ukin"] = ukin
        v["Uelm"] = float(np.sum(fe))
        v["Utot"] = v["Ukin"] + v["Uelm"] + v["Urad"]
        if itime == 0:
            self.energy_time_zero = v["Utot"]
        v["Uexp"] = self.energy_time_zero
        v["Ubal"] = v["Utot"] - v["Uexp"]
        v["Ubal_norm"] = v["Ubal"] / v["Utot"] if v["Utot"] > 0.0 else 0.0
        for f in MINMAX_FIELDS:
            if not (self._allowed(f + "Min") or self._allowed(f + "Max")):
                continue
            a = self._interior(sim.rho() if f == "Rho" else sim.get_field(f)).astype(np.float64)
            flat = a.ravel()  # C order: i * N1 * N2 + j * N2 + k
            imin, imax = int(np.argmin(flat)), int(np.argmax(flat))
            v[f + "Min"], v[f + "MinCell"] = float(flat[imin]), imin
            v[f + "Max"], v[f + "MaxCell"] = float(flat[imax]), imax
        for a in "XYZ"[: sim.ndim]:
            for side in ("min", "max"):
                v[f"Poy{a}{side}"] = 0.0  # no flux through periodic boundaries
                v[f"Poy{a}{side}Inst"] = 0.0
        return v

    # ---- file ---------------------------------------------------------------------
    def header(self) -> str:
        p = self.precision
        lines = ["# 1 time"]
        j = 2
        for name, second in self.columns():
            lines.append(f"# {j} {name}")
            j += 1
            if second:
                lines.append(f"# {j} {second}")
                j += 1
        row = "#" + f"{'time':>{p + 9}}"
        for name, second in self.columns():
            w = column_width(name, p)
            row += f"{name:>{w}}"
            if second:
                row += f"{second:>{w}}"
        return "\n".join(lines) + "\n#\n" + row + "\n"

    def row(self, itime: int, values: dict) -> str:
        p = self.precision
        out = _sci(itime * self.sim.dt, p, p + 10)
        for name, second in self.columns():
            w = column_width(name, p)
            out += _sci(values[name], p, w)
            if second:
                out += f"{int(values[second]):>{w}d}"
        return out + "\n"

    def __call__(self, itime: int):
        """Writes the row of step ``itime`` when it is a diagnostic step (and not written yet)."""
        if itime % self.every or itime <= self.latest:
            return None
        vals = self.values(itime)
        mode = "a" if self._header_written else "w"
        with open(self.path, mode) as f:
            if not self._header_written:
                f.write(self.header())
                self._header_written = True
            f.write(self.row(itime, vals))
        self.latest = itime
        return vals


def read_scalars(path: str) -> dict:
    """Columns of a scalars.txt (this module's or the reference's) as numpy arrays by name."""
    names = []
    rows = []
    with open(path) as f:
        for line in f:
            if line.startswith("#"):
                parts = line[1:].split()
                if len(parts) == 2 and parts[0].isdigit():
                    names.append(parts[1])
                continue
            if line.strip():
                rows.append([float(x) for x in line.split()])
    data = np.array(rows, dtype=np.float64).reshape(len(rows), len(names)) if rows else np.zeros((0, len(names)))
    return {n: data[:, i] for i, n in enumerate(names)}


FIELD_NAMES = ["Ex", "Ey", "Ez", "Bx", "By", "Bz", "Bx_m", "By_m", "Bz_m", "Jx", "Jy", "Jz", "Rho"]


class DiagFields:
    """Field dumps in the reference's DiagFields layout, as .npz instead of HDF5.

    The reference (src/Diagnostic/DiagnosticFields2D.cpp:20-55,150-190 and its 3D
    twin) writes, for every field whatever its staggering, the N + 1 points per
    dimension that start at array index oversize (the patches' own points, the
    first patch contributing its lower border), into group ``data/<itime>`` of
    Fields<n>.h5 with the attribute ``x_moved``.  Here each dump is one file
    ``<path>/<itime>.npz`` holding one array per field and ``x_moved``;
    ``time_average`` = T > 1 sums the fields of the T steps that start at each
    selected step k * every and writes their sum times 1/T at step k * every + T - 1
    (DiagnosticFields::prepare and run, src/Diagnostic/DiagnosticFields.cpp:262-292);
    ``subgrid`` is a tuple of slices applied to the dumped (N + 1)-point arrays."""

    def __init__(self, sim, path="Fields0", every=1, fields=None, time_average=1, subgrid=None):
        import os
        self.sim = sim
        self.path = path
        self.every = int(every)
        self.fields = list(fields) if fields else [f for f in FIELD_NAMES if f != "Rho"]
        self.time_average = max(1, int(time_average))
        self.subgrid = subgrid
        self._acc = {}
        os.makedirs(path, exist_ok=True)

    def _grab(self, name):
        a = self.sim.rho() if name == "Rho" else self.sim.get_field(name)
        nd = len(self.sim.n_cells)
        sl = tuple(slice(OVERSIZE, OVERSIZE + self.sim.n_cells[d] + 1) for d in range(nd))
        out = np.ascontiguousarray(a[sl])
        return out[self.subgrid] if self.subgrid is not None else out

    def __call__(self, itime: int):
        """Accumulates (time average) and writes the dump of step ``itime`` when it is due."""
        phase = itime % self.every
        if phase >= self.time_average:
            return None
        if self.time_average > 1:
            for f in self.fields:
                self._acc[f] = self._acc.get(f, 0.0) + self._grab(f)
            if phase != self.time_average - 1:
                return None
            inv = 1.0 / self.time_average
            data = {f: self._acc[f] * inv for f in self.fields}
            self._acc = {}
        else:
            data = {f: self._grab(f) for f in self.fields}
        x_moved = self.sim.window_state()[1] if hasattr(self.sim, "window_state") else 0.0
        import os
        np.savez(os.path.join(self.path, f"{itime}.npz"), x_moved=np.float64(x_moved), **data)
        return data


def read_fields(path: str) -> dict:
    """{itime: {field: array, "x_moved": float}} of a DiagFields directory."""
    import os
    out = {}
    for fn in os.listdir(path):
        if fn.endswith(".npz") and fn[:-4].isdigit():
            z = np.load(os.path.join(path, fn))
            out[int(fn[:-4])] = {k: (float(z[k]) if k == "x_moved" else z[k]) for k in z.files}
    return dict(sorted(out.items()))


__all__ = ["DiagScalar", "read_scalars", "column_width", "GENERAL", "SPECIES", "ENERGY_FIELDS", "MINMAX_FIELDS",
           "DiagFields", "read_fields", "FIELD_NAMES"]
