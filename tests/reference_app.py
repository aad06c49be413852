"""The reference phonomena application with the GB300 plugin, in a fresh interpreter.

Test infrastructure.  ``python tests/reference_app.py MODE OUTDIR`` copies the
reference application (the baseline/_ref install, or $PHONO_REFERENCE_ROOT)
to OUTDIR/app, installs the stand-ins of oracle/ref_harness.install_shims
with tests/h5shim.py as h5py, and runs the application's own code paths:

* ``common.findSolvers()`` (phonomena/common.py:93-110) over a solvers
  directory to which ``solver_gb300.py`` was added (a two-line module that
  re-exports ``phonomena_gb300.solver_gb300``: INTEGRATION.md's recipe);
* ``common.loadSettings()`` (phonomena/common.py:112-156) on the
  application's own data/default.json (GaAs with six Au inclusions), with
  ``"solver"`` set to the plugin's name, which selects the plugin;
* the reference's ``solver_default`` with its own Writer (write_mode
  'thread', through the h5py stand-in), and ``analysis.spectrum``
  (simulation/analysis.py:44-96) on every file.

MODE ``gpu`` runs the plugin twice on the GPU (surface records every 5
steps; the full volume after every step); MODE ``schema`` (no GPU) writes
the plugin's file format from the reference solver's own results through
phonomena_gb300.output, to check the schema alone.  Results go to
OUTDIR/result.npz; the tests compare them.
"""
from __future__ import annotations

import json
import shutil
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
STEPS = 40        # the default_json golden fixture's length
RECORD_EVERY = 5  # and its surface-record period
Y_INDEX = 7       # a y row through two inclusions


def _spectrum_args():
    return [("uz", dict(z_index=0, y_index=Y_INDEX)), ("uz", dict(z_index=0, y_index=Y_INDEX, x_index=20))]


def _volume_spectrum_args():
    return [("ux", dict(z_index=2, y_index=Y_INDEX)), ("uy", dict(z_index=1, y_index=Y_INDEX, x_index=10)),
            ("uz", dict(z_index=1, y_index=Y_INDEX))]


def setup(outdir):
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "tests"))
    import h5shim
    from oracle import ref_harness as H

    if not H.available():
        raise SystemExit(f"reference application not installed under {H.REF_ROOT}")
    app = Path(outdir) / "app"
    if app.exists():
        shutil.rmtree(app)
    shutil.copytree(H.REF_ROOT / "phonomena", app / "phonomena")
    shutil.copytree(H.REF_ROOT / "data", app / "data")
    (app / "phonomena" / "simulation" / "solvers" / "solver_gb300.py").write_text(
        '"""GB300 (sm_103a) solver: phonomena_gb300\'s plugin in this registry."""\n'
        "from phonomena_gb300.solver_gb300 import Solver, cfg  # noqa: F401\n")
    settings = json.loads((app / "data" / "default.json").read_text())
    settings["simulation"]["solver"] = "gb300"
    (app / "data" / "gb300.json").write_text(json.dumps(settings))
    H.install_shims(h5py_module=h5shim)
    sys.path.insert(0, str(app))
    from phonomena import common  # noqa: E402  (appends phonomena/ to sys.path)

    return app, common


def reference_file(common, grid, material, outdir):
    """The reference solver_default's own result file (every step, full volume),
    with the settings file's solver cfg (sin source, 100 Hz)."""
    s = common.solver_dict["default"]
    s.cfg = {**s.cfg, **common.cfg["simulation"]["cfg"], "write_mode": "thread"}
    s.file = str(Path(outdir) / "reference.h5")
    s.init(grid, material, STEPS)
    s.run()
    return s


def sampled_copy(src, dst, k):
    """The reference file with its time axis kept at steps k-1, 2k-1, ... and
    attrs dt multiplied by k: what a writer sampling every k-th step stores."""
    import h5py  # the stand-in

    with h5py.File(src, "r") as a, h5py.File(dst, "w") as b:
        for name in ("ux", "uy", "uz"):
            b.create_dataset(name, data=a[name][..., k - 1::k])
        for key, v in a.attrs.items():
            b.attrs[key] = v
        b.attrs["dt"] = float(a.attrs["dt"]) * k
    return dst


def spectra(analysis, path, args):
    out = {}
    for q, (u_id, kw) in enumerate(args):
        x, f, dft = analysis.spectrum(str(path), u_id, **kw)
        out[f"s{q}_x"], out[f"s{q}_f"], out[f"s{q}_dft"] = np.asarray(x), np.asarray(f), np.asarray(dft)
    return out


def main(mode, outdir):
    outdir = Path(outdir)
    outdir.mkdir(parents=True, exist_ok=True)
    app, common = setup(outdir)
    common.findSolvers()
    _, grid, material = common.loadSettings(str(app / "data" / "gb300.json"))
    from simulation import analysis, base_solver  # the application's own modules

    res = {"found": np.array(sorted(common.solver_dict)), "selected": np.array(common.solver.name)}
    ref = reference_file(common, grid, material, outdir)
    ref_sampled = sampled_copy(ref.file, str(outdir / "reference_sampled.h5"), RECORD_EVERY)
    res.update({f"ref_{k}": v for k, v in spectra(analysis, ref_sampled, _spectrum_args()).items()})
    res.update({f"refvol_{k}": v for k, v in spectra(analysis, ref.file, _volume_spectrum_args()).items()})
    res["ref_ux"], res["ref_uy"], res["ref_uz"] = ref.g.ux, ref.g.uy, ref.g.uz
    sec = np.array(ref.m.secondary["c"])
    res["ref_secondary"] = (np.all(ref.m.C == sec, axis=(-1, -2)) & (ref.m.P == float(ref.m.secondary["p"])))

    if mode == "gpu":
        plugin = common.solver
        res["subclass"] = np.array(isinstance(plugin, base_solver.BaseSolver))
        plugin.cfg.update(record_every=RECORD_EVERY, output="surface", write_mode="process")
        plugin.file = str(outdir / "gb300_surface")
        plugin.init(grid, material, STEPS)
        progress = []

        class Sig:
            class _S:
                def __init__(self, sink):
                    self.sink = sink

                def emit(self, v):
                    self.sink.append(v)

            def __init__(self):
                self.status, self.progress = Sig._S([]), Sig._S(progress)

        plugin.run(signals=Sig())
        res["progress"] = np.array(progress)
        res["ux"], res["uy"], res["uz"], res["surf"] = plugin.g.ux, plugin.g.uy, plugin.g.uz, plugin.surface
        res["ids"] = plugin.material_ids()
        res["file_surface"] = np.array(plugin.file)
        res.update({f"gb_{k}": v for k, v in spectra(analysis, plugin.file, _spectrum_args()).items()})
        plugin.cfg.update(record_every=1, output="volume")
        plugin.file = str(outdir / "gb300_volume")
        plugin.init(grid, material, STEPS)
        plugin.run()
        res.update({f"gbvol_{k}": v for k, v in spectra(analysis, plugin.file, _volume_spectrum_args()).items()})
        plugin.release()
    else:  # schema: the plugin's writer on the reference solver's own results
        from phonomena_gb300 import output

        class Done:  # a finished GB300 run holding the reference's results
            def __init__(self, g, m, cfg, record_every, surface=None, volume=None):
                self.g, self.m, self.cfg, self.t = g, m, cfg, STEPS
                self.record_every, self.surface, self.volume = record_every, surface, volume
                ids = np.zeros(g.x.size * g.y.size * g.z.size, np.uint8).reshape(g.x.size, g.y.size, g.z.size)
                ids[res["ref_secondary"]] = 1
                self._ids = ids

            def material_ids(self):
                return self._ids

            def material_table(self):
                from phonomena_gb300.model import table_row

                return np.stack([table_row(self.m.primary["c"], self.m.primary["p"]),
                                 table_row(self.m.secondary["c"], self.m.secondary["p"])])

        import h5py  # the stand-in

        with h5py.File(ref.file, "r") as f:
            full = {k: np.array(f[k][...]) for k in ("ux", "uy", "uz")}
        surf = np.moveaxis(full["uz"][:, :, 0, RECORD_EVERY - 1::RECORD_EVERY], 2, 0)
        path = output.write_results(str(outdir / "schema_surface"), Done(ref.g, ref.m, {}, RECORD_EVERY, surf))
        res.update({f"gb_{k}": v for k, v in spectra(analysis, path, _spectrum_args()).items()})
        path = output.write_results(str(outdir / "schema_volume"), Done(ref.g, ref.m, {}, 1, volume=full))
        res.update({f"gbvol_{k}": v for k, v in spectra(analysis, path, _volume_spectrum_args()).items()})
    np.savez(outdir / "result.npz", **res)


if __name__ == "__main__":
    main(sys.argv[1], sys.argv[2])
