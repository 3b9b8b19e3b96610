"""Recipe: compile the reference's CPU PBR builder into ``oracle/_ref/``.

Test infrastructure only.  Nothing in the product imports this module.

It compiles two source files of the reference, where they lie under the
read-only reference checkout, into a CPU-only Python extension named
``graph_link_core``:

* ``Backend/graph_link/pbr_matrix/pbr_matrix.cpp`` (``csr_to_pbr``,
  ``pbr_to_csr``, the CPU SpMM);
* ``Backend/graph_link/bindings/bindings.cpp`` (the pybind11 module and the
  ``PBRMatrix*`` property getters).

``CUDA_ENABLED`` is left undefined, so no ``.cu`` file is involved.  The
reference's own ``setup.py`` is not run (it fails on current setuptools); the
two files are handed to ``torch.utils.cpp_extension.load`` with the flags the
reference uses for its host code (``-O3 -std=c++20 -w``).  Torch supplies the
ATen and pybind11 headers the two files include.

The compiled module is the ground truth the C++ restatement in
``oracle/pbr_oracle.cpp`` is checked against, and the generator of the golden
fixtures under ``tests/golden/``.  It only exists where the reference checkout
exists; the GPU machines never build it.

Usage::

    python oracle/ref_build.py          # builds oracle/_ref/graph_link_core*.so

The reference checkout is taken from ``$GL_REFERENCE_ROOT`` or, when that is
unset, from a directory named ``reference`` beside this repository.
"""
from __future__ import annotations

import importlib.util
import os
import sys
from pathlib import Path

def _reference_root() -> Path:
    """The reference checkout: $GL_REFERENCE_ROOT, else a directory named
    ``reference`` beside this repository's directory."""
    env = os.environ.get("GL_REFERENCE_ROOT")
    if env:
        return Path(env)
    return Path(__file__).resolve().parents[2] / "reference"


REFERENCE_ROOT = _reference_root()
REF_SRC = REFERENCE_ROOT / "Backend" / "graph_link"
OUT_DIR = Path(__file__).resolve().parent / "_ref"


def reference_present() -> bool:
    return (REF_SRC / "pbr_matrix" / "pbr_matrix.cpp").is_file()


def built_module_path() -> Path | None:
    if not OUT_DIR.is_dir():
        return None
    for p in sorted(OUT_DIR.glob("graph_link_core*.so")):
        return p
    return None


def build(verbose: bool = False) -> Path | None:
    """Compile the reference builder if the reference checkout is present."""
    if not reference_present():
        return None
    existing = built_module_path()
    if existing is not None:
        return existing
    from torch.utils.cpp_extension import load

    OUT_DIR.mkdir(parents=True, exist_ok=True)
    build_dir = OUT_DIR / "build"
    build_dir.mkdir(exist_ok=True)
    load(
        name="graph_link_core",
        sources=[str(REF_SRC / "bindings" / "bindings.cpp"),
                 str(REF_SRC / "pbr_matrix" / "pbr_matrix.cpp")],
        extra_cflags=["-O3", "-std=c++20", "-w"],
        extra_include_paths=[str(REF_SRC)],
        build_directory=str(build_dir),
        verbose=verbose,
        is_python_module=True,
        with_cuda=False,
    )
    so = next(build_dir.glob("graph_link_core*.so"))
    target = OUT_DIR / so.name
    target.write_bytes(so.read_bytes())
    return target


def load_reference_core():
    """Import the compiled reference builder, or return None when absent."""
    path = built_module_path()
    if path is None:
        return None
    import torch  # noqa: F401  (loads libc10 / libtorch the module links against)
    spec =importlib.util.spec_from_file_location("graph_link_core", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


if __name__ == "__main__":
    out = build(verbose="-v" in sys.argv)
    print(out if out is not None else "reference sources not present; nothing built")
