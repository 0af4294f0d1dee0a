"""Install the unmodified reference (nanodrr) into baseline/_ref for the
reference-kernel legs of bench.py and tests/test_reference_triton_gpu.py.

The offline `pip install --target baseline/_ref <checkout>` cannot run: the
reference's build backend (uv_build) is not in the wheelhouse. The package is
pure Python, so its `src/nanodrr` is copied as is. Four of its third-party
imports are absent from this image and the GPU hosts: jaxtyping (annotations),
torchio (file loading), roma (rotation conversions) and platformdirs (demo
data); the stand-ins of tests/golden/_refstubs, which none of the rendering
arithmetic touches, are copied beside it.

Usage: python baseline/install_reference.py /path/to/nanodrr-checkout
(or NANODRR_REFERENCE=/path/to/nanodrr-checkout).
"""

from __future__ import annotations

import os
import shutil
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
DEST = HERE / "_ref"


def main() -> None:
    src = Path(sys.argv[1]) if len(sys.argv) > 1 else Path(os.environ.get("NANODRR_REFERENCE", ""))
    pkg = src / "src" / "nanodrr"
    if not pkg.is_dir():
        sys.exit("usage: install_reference.py /path/to/nanodrr-checkout (its src/nanodrr was not found)")
    if DEST.exists():
        shutil.rmtree(DEST)
    DEST.mkdir(parents=True)
    shutil.copytree(pkg, DEST / "nanodrr", ignore=shutil.ignore_patterns("__pycache__", "*.pyc"))
    for stub in sorted((REPO / "tests" / "golden" / "_refstubs").iterdir()):
        if stub.is_dir():
            shutil.copytree(stub, DEST / stub.name, ignore=shutil.ignore_patterns("__pycache__", "*.pyc"))
    (DEST / "INSTALLED_FROM").write_text(f"{src.resolve()}\n")
    print(f"installed {pkg} -> {DEST / 'nanodrr'} (+ stand-ins for jaxtyping, torchio, roma, platformdirs)")


if __name__ == "__main__":
    main()
