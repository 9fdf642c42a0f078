"""In-tree build of ``libquiqbox_gb300.so`` for sm_103a.

Steps: generate the ERI class kernels (csrc/gen_eri.py) into ``_build/gen``,
compile every CUDA translation unit in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo`` and link the
shared library ``_build/libquiqbox_gb300.so`` (CUDA runtime linked statically,
so the library loads without a toolkit on the library path).
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
GEN = OUT / "gen"
OBJ = OUT / "obj"
INCLUDE = PKG.parent / "include"
LIB = OUT / "libquiqbox_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HAND_WRITTEN = ["engine.cu", "generic.cu", "linalg.cu", "scf.cu", "capi.cu", "noalloc.cu", "batch.cu", "mlp.cu", "guess.cu"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _headers():
    return list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))


def _stale(obj: Path, deps):
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose=False, jobs=None):
    OUT.mkdir(exist_ok=True)
    OBJ.mkdir(exist_ok=True)
    gen_script = CSRC / "gen_eri.py"
    marker = GEN / "eri_dispatch.cu"
    if not marker.exists() or marker.stat().st_mtime < gen_script.stat().st_mtime:
        subprocess.run([sys.executable, str(gen_script), str(GEN)], check=True, stdout=subprocess.DEVNULL)
    nvcc = _nvcc()
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-warn-spills",
                    f"-I{CSRC}", f"-I{GEN}", f"-I{INCLUDE}"]
    hdrs = _headers()
    units = [(CSRC / s, [CSRC / s] + hdrs) for s in HAND_WRITTEN]
    for cu in sorted(GEN.glob("eri_class_*.cu")) + [GEN / "eri_dispatch.cu"]:
        deps = [cu] + hdrs
        cuh = cu.with_suffix(".cuh")
        if cuh.exists():
            deps.append(cuh)
        units.append((cu, deps))
    # heaviest translation units first
    units.sort(key=lambda u: -u[0].stat().st_size)

    def compile_one(unit):
        src, deps = unit
        obj = OBJ / (src.stem + ".o")
        if not _stale(obj, deps):
            return None
        cmd = [nvcc] + flags + ["-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            return f"{src.name}:\n{r.stdout}\n{r.stderr}"
        if verbose:
            print(src.name, r.stderr.strip()[-400:])
        return None

    jobs = jobs or max(1, os.cpu_count() or 1)
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        errs = [e for e in ex.map(compile_one, units) if e]
    if errs:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errs))
    objs = [OBJ / (u[0].stem + ".o") for u in units]
    if _stale(LIB, objs):
        cmd = [nvcc] + ARCH + ["-shared", "-o", str(LIB)] + [str(o) for o in objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
