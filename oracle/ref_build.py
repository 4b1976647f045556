"""Build the reference's own CPU code for the closure path, from its sources in place.

Test infrastructure only (oracle pinning).  This recipe compiles the three native
pieces of redblackgraph that the closure path runs on the CPU:

* ``redblackgraph.core._redblackgraph``      -- C: ``warshall`` gufunc, AVOS einsum,
  scalar ``avos_sum``/``avos_product`` (sources per ``redblackgraph/core/meson.build``);
* ``redblackgraph.sparse._sparsetools``      -- C++: ``rbm_matmat_pass1/pass2``
  (``redblackgraph/sparse/meson.build``);
* ``redblackgraph.sparse.csgraph._*``         -- Cython: ``floyd_warshall``, DAG closure,
  components, topological sort (``redblackgraph/sparse/csgraph/meson.build``).

Templates are expanded with ``Cython.Tempita`` (a drop-in for the ``tempita`` package that
``tools/tempita_processor.py`` imports) and the reference's own
``tools/process_src_template.py``.  Generated C and compiled modules go only into
``oracle/_ref/``; the reference's Python sources are imported from where they lie through
:mod:`oracle.refimport`.  The reference is read, never copied into the repository.

Run here (x86 container, where the reference is mounted):  ``python oracle/ref_build.py``.
The GPU host has no reference tree; nothing there depends on this script.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys
import sysconfig
from pathlib import Path

REF_ROOT = Path(os.environ.get("RBG_REFERENCE_ROOT", "/root/reference"))
HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
GEN = OUT / "gen"
PKG = OUT / "redblackgraph"


def _numpy_include() -> str:
    import numpy
    return numpy.get_include()


def _py_include() -> str:
    return sysconfig.get_paths()["include"]


def _ext_suffix() -> str:
    return sysconfig.get_config_var("EXT_SUFFIX")


def _run(cmd, **kw):
    r = subprocess.run(cmd, capture_output=True, text=True, **kw)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")
    return r


def _tempita(src: Path, dst: Path) -> None:
    from Cython import Tempita
    text = src.read_text(encoding="utf-8")
    dst.parent.mkdir(parents=True, exist_ok=True)
    dst.write_text(Tempita.Template(text, name=str(src)).substitute(), encoding="utf-8")


def _stale(out: Path, *inputs: Path) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(p.stat().st_mtime > t for p in inputs)


def build_core() -> Path:
    src = REF_ROOT / "redblackgraph" / "core" / "src" / "redblackgraph"
    gen = GEN / "core"
    gen.mkdir(parents=True, exist_ok=True)
    for name in ("rbg_math.h", "rbg_math.c", "warshall.c", "relational_composition.c"):
        _tempita(src / (name + ".in"), gen / name)
    _run([sys.executable, str(REF_ROOT / "tools" / "process_src_template.py"),
          str(src / "redblack.c.src"), "-o", str(gen / "redblack.c")])
    out = PKG / "core" / ("_redblackgraph" + _ext_suffix())
    out.parent.mkdir(parents=True, exist_ok=True)
    sources = [src / "redblackgraphmodule.c", gen / "rbg_math.c", gen / "redblack.c",
               gen / "relational_composition.c", gen / "warshall.c"]
    _run(["gcc", "-O2", "-fPIC", "-shared", "-w",
          "-DNPY_NO_DEPRECATED_API=NPY_1_7_API_VERSION",
          f"-I{_numpy_include()}", f"-I{_py_include()}", f"-I{src}", f"-I{gen}",
          f"-I{REF_ROOT / 'redblackgraph' / 'core' / 'include'}",
          *map(str, sources), "-o", str(out)])
    return out


def build_sparsetools() -> Path:
    src = REF_ROOT / "redblackgraph" / "sparse" / "sparsetools"
    out = PKG / "sparse" / ("_sparsetools" + _ext_suffix())
    out.parent.mkdir(parents=True, exist_ok=True)
    _run(["g++", "-O2", "-fPIC", "-shared", "-w", "-std=c++14",
          "-D__STDC_FORMAT_MACROS=1", "-DNPY_NO_DEPRECATED_API=NPY_1_7_API_VERSION",
          f"-I{_numpy_include()}", f"-I{_py_include()}", f"-I{src}",
          str(src / "sparsetools.cxx"), str(src / "rbm.cxx"), "-o", str(out)])
    return out


CYTHON_MODULES = ("_shortest_path", "_rbg_math", "_components", "_permutation", "_ordering",
                  "_relational_composition", "_tools", "_topological_sort",
                  "_transitive_closure_dag")


def _build_cython(name: str) -> Path:
    src_dir = REF_ROOT / "redblackgraph" / "sparse" / "csgraph"
    gen = GEN / "csgraph"
    gen.mkdir(parents=True, exist_ok=True)
    c_file = gen / (name + ".c")
    _run([sys.executable, "-m", "cython", "-3", "-I", str(src_dir), "-o", str(c_file),
          str(src_dir / (name + ".pyx"))])
    out = PKG / "sparse" / "csgraph" / (name + _ext_suffix())
    out.parent.mkdir(parents=True, exist_ok=True)
    _run(["gcc", "-O2", "-fPIC", "-shared", "-w",
          "-DNPY_NO_DEPRECATED_API=NPY_1_7_API_VERSION",
          f"-I{_numpy_include()}", f"-I{_py_include()}", f"-I{src_dir}",
          str(c_file), "-o", str(out)])
    return out


def build(force: bool = False) -> bool:
    """Build every reference extension on the path; return False when no reference tree."""
    if not (REF_ROOT / "redblackgraph").is_dir():
        return False
    marker = OUT / ".built"
    if marker.exists() and not force:
        return True
    OUT.mkdir(parents=True, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        futs = [ex.submit(build_core), ex.submit(build_sparsetools)]
        futs += [ex.submit(_build_cython, n) for n in CYTHON_MODULES]
        for f in futs:
            f.result()
    marker.write_text("ok\n")
    return True


if __name__ == "__main__":
    ok = build(force="--force" in sys.argv)
    print("reference built into", OUT if ok else "(no reference tree)")
