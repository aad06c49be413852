"""Install the reference phonomena application into baseline/_ref/.

TEST AND BENCHMARK INFRASTRUCTURE ONLY.  phonomena is a pure-Python
application without a package build: its ``setup.py`` is an installer script
that runs ``pip install matplotlib PyQt5 numpy h5py numba ...`` from an
index, so ``pip install --target`` fails at metadata generation.  The install
is therefore a copy of the application's Python sources and settings files:

    <reference>/phonomena/**.py   -> baseline/_ref/phonomena/
    <reference>/data/*.json       -> baseline/_ref/data/
    <reference>/tests/data/*.json -> baseline/_ref/tests/data/

Usage (from the repository root):

    python oracle/install_reference.py [REFERENCE_ROOT]

REFERENCE_ROOT defaults to $PHONO_REFERENCE_ROOT, else /root/reference.
baseline/_ref/ is listed in .gitignore (no reference source enters the
repository's history) and travels with the working tree to the GPU machine,
where the tests and bench.py's reference arm import it with the shims of
oracle/ref_harness.py.
"""
from __future__ import annotations

import os
import shutil
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
DEST = ROOT / "baseline" / "_ref"


def install(src: Path | str | None = None, dest: Path = DEST) -> Path:
    src = Path(src or os.environ.get("PHONO_REFERENCE_ROOT", "/root/reference"))
    if not (src / "phonomena" / "simulation" / "base_solver.py").exists():
        raise FileNotFoundError(f"no phonomena sources under {src}")
    if dest.exists():
        shutil.rmtree(dest)
    dest.mkdir(parents=True)
    for rel in ("phonomena",):
        for p in sorted((src / rel).rglob("*.py")):
            out = dest / p.relative_to(src)
            out.parent.mkdir(parents=True, exist_ok=True)
            shutil.copyfile(p, out)
    for rel in ("data", "tests/data"):
        for p in sorted((src / rel).glob("*.json")):
            out = dest / p.relative_to(src)
            out.parent.mkdir(parents=True, exist_ok=True)
            shutil.copyfile(p, out)
    (dest / "INSTALLED_FROM").write_text(str(src) + "\n")
    return dest


if __name__ == "__main__":
    print(install(sys.argv[1] if len(sys.argv) > 1 else None))
