"""Build recipe for the sm_103a SPH step library and its host-side companions.

  libsphx.so        CUDA kernels + C ABI (include/sphx.h)        -> <pkg>/lib/
  libsph_gb300.so   C++17 drop-in SPHEngine over the C ABI       -> <pkg>/lib/
  sph*.so           pybind11 module `sph` over the drop-in       -> <pkg>/lib/
  oracle (tests)    oracle/_build/libsph_oracle.so, and oracle/_ref/libsph_ref.so when the
                    reference sources are present (oracle/build_ref.sh)

Every translation unit is compiled in parallel with one -gencode (sm_103a); host code is
built with -ffp-contract=off so float expressions round exactly as written.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
import sysconfig
from pathlib import Path

PKG = Path(__file__).resolve().parents[1]
REPO = PKG.parent
LIB = PKG / "lib"
OBJ = PKG / "_build"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler",
              "-ffp-contract=off", "-Xptxas", "-warn-spills", f"-I{REPO / 'include'}"]
CUDA_SOURCES = ["sphx_sort.cu", "sphx_grid.cu", "sphx_passes.cu", "sphx_density.cu",
                "sphx_force.cu", "sphx_sweep.cu", "sphx_batch.cu",
                "sphx_capi.cu", "sphx_hash.cu", "sphx_noalloc.cu",
                "sphx_render.cu", "sphx_gen.cu"]


def _nvcc() -> str:
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = Path(home) / "bin" / "nvcc"
    return str(cand) if cand.exists() else (shutil.which("nvcc") or "nvcc")


def _run_parallel(cmds: list[list[str]]) -> None:
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for c in cmds]
    errors = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append(f"$ {' '.join(c)}\n{out.decode(errors='replace')}")
        elif out.strip():
            sys.stderr.write(out.decode(errors="replace"))
    if errors:
        raise RuntimeError("build failed:\n" + "\n".join(errors))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_sphx(force: bool = False) -> Path:
    """Compiles the CUDA library; returns the .so path."""
    LIB.mkdir(exist_ok=True)
    OBJ.mkdir(exist_ok=True)
    csrc = PKG / "csrc"
    headers = list(csrc.glob("*.cuh")) + [REPO / "include" / "sphx.h"]
    nvcc = _nvcc()
    cmds, objs = [], []
    for s in CUDA_SOURCES:
        src, obj = csrc / s, OBJ / (Path(s).stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmds.append([nvcc, *NVCC_FLAGS, *ARCH, "-c", str(src), "-o", str(obj)])
    _run_parallel(cmds)
    so = LIB / "libsphx.so"
    if force or cmds or _stale(so, objs):
        _run_parallel([[nvcc, "-shared", *ARCH, "-o", str(so), *map(str, objs)]])
    return so


HOST_SOURCES = ["kernels.cpp", "particle.cpp", "spatial_hash.cpp", "sph_engine.cpp"]
HOST_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fopenmp", "-Wall", "-Wextra",
              f"-I{REPO / 'include'}", f"-I{PKG / 'host' / 'include'}",
              "-idirafter", str(PKG / "host" / "compat")]


def build_host(force: bool = False) -> Path:
    """Compiles the C++17 drop-in engine (SPHEngine, ParticleSystem, SpatialHash) into
    libsph_gb300.so, linked against libsphx.so."""
    sphx = build_sphx(force)
    srcs = [PKG / "host" / "src" / s for s in HOST_SOURCES]
    deps = srcs + list((PKG / "host" / "include").glob("*.h")) + [REPO / "include" / "sphx.h", sphx]
    so = LIB / "libsph_gb300.so"
    if force or _stale(so, deps):
        _run_parallel([["g++", *HOST_FLAGS, "-shared", *map(str, srcs), f"-L{LIB}", "-lsphx",
                        "-Wl,-rpath,$ORIGIN", "-o", str(so)]])
    return so


def _pybind_include() -> str | None:
    import importlib.util

    spec = importlib.util.find_spec("torch")
    if spec and spec.submodule_search_locations:
        inc = Path(list(spec.submodule_search_locations)[0]) / "include"
        if (inc / "pybind11" / "pybind11.h").exists():
            return str(inc)
    try:
        import pybind11

        return pybind11.get_include()
    except ImportError:
        return None


def build_pymodule(force: bool = False) -> Path | None:
    """Compiles the pybind11 module `sph` (the reference's Python API) into <pkg>/lib."""
    host = build_host(force)
    pyinc = sysconfig.get_paths()["include"]
    pbinc = _pybind_include()
    if not (Path(pyinc) / "Python.h").exists() or not pbinc:
        sys.stderr.write("sph module not built: Python.h or pybind11 headers missing\n")
        return None
    src = PKG / "python" / "sph_module.cpp"
    so = LIB / ("sph" + sysconfig.get_config_var("EXT_SUFFIX"))
    if force or _stale(so, [src, host]):
        _run_parallel([["g++", *HOST_FLAGS, "-shared", f"-I{pyinc}", f"-I{pbinc}", str(src),
                        f"-L{LIB}", "-lsph_gb300", "-lsphx", "-Wl,-rpath,$ORIGIN", "-o", str(so)]])
    return so


def build_oracle(force: bool = False) -> Path:
    """Compiles the C restatement of the reference step (test infrastructure)."""
    out_dir = REPO / "oracle" / "_build"
    out_dir.mkdir(exist_ok=True)
    srcs = [REPO / "oracle" / "sph_oracle.c", REPO / "oracle" / "render_oracle.c"]
    so = out_dir / "libsph_oracle.so"
    if force or _stale(so, srcs + [REPO / "oracle" / "sph_oracle.h"]):
        _run_parallel([["gcc", "-std=c11", "-D_GNU_SOURCE", "-O2", "-fopenmp",
                        "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
                        *map(str, srcs), "-o", str(so), "-lm"]])
    return so


def build_ref() -> Path | None:
    """Builds oracle/_ref from the reference sources when they are present (their location:
    SPH_REFERENCE_DIR, else the default of oracle/build_ref.sh); None when they are not."""
    so = REPO / "oracle" / "_ref" / "libsph_ref.so"
    deps = [REPO / "oracle" / "ref_harness.cpp", REPO / "oracle" / "glm_shim" / "glm" / "glm.hpp",
            REPO / "oracle" / "build_ref.sh"]
    if not _stale(so, deps):
        return so
    cmd = ["bash", str(REPO / "oracle" / "build_ref.sh")]
    if os.environ.get("SPH_REFERENCE_DIR"):
        cmd.append(os.environ["SPH_REFERENCE_DIR"])
    r = subprocess.run(cmd, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, text=True)
    if r.returncode == 2:  # no reference checkout on this machine
        return None
    if r.returncode != 0:
        raise RuntimeError("reference build failed:\n" + r.stderr)
    return so


def build_all(force: bool = False) -> dict:
    out = {"sphx": build_sphx(force), "oracle": build_oracle(force)}
    out["host"] = build_host(force)
    out["sph_module"] = build_pymodule(force)
    out["ref"] = build_ref()
    return out


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv))
