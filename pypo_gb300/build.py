"""Build libpo_gb300.so in-tree with nvcc for sm_103a (no cmake).

The translation units compile in parallel; the link uses the shared CUDA
runtime so that device pointers and streams are shared with PyTorch.
"""
import concurrent.futures
import os
import pathlib
import shutil
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
CSRC = HERE / "csrc"
INCLUDE = HERE.parent / "include"
LIB = HERE / "libpo_gb300.so"
BUILD = HERE / "_build"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["po_kernels.cu", "po_farfield.cu", "po_adjoint.cu", "po_adjoint_pk.cu", "po_engine.cu", "po_capi.cu", "po_grid.cpp", "po_grid_dev.cu", "po_sources_dev.cu", "po_eff_dev.cu", "po_noalloc.cu", "po_fmin.cpp", "po_fitgauss_dev.cu"]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libpo_gb300")
    return path


def _compile(src, verbose=False, defines=(), build_dir=None):
    obj = (build_dir or BUILD) / (src + ".o")
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3,-ffp-contract=off",
           *[f"-D{d}" for d in defines], "-I", str(INCLUDE), "-c", str(CSRC / src), "-o", str(obj)]
    if verbose and src.endswith(".cu"):
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build_variant(out_path, defines, verbose=False):
    """Build a copy of the library with PO_* tuning macros into out_path (tuning sweeps)."""
    out_path = pathlib.Path(out_path)
    bdir = out_path.parent / (out_path.stem + "_obj")
    bdir.mkdir(parents=True, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose, defines, bdir), SOURCES))
    cmd = [nvcc(), *ARCH, "-shared", "-cudart", "shared", "-o", str(out_path), *[str(o) for o, _ in results],
           "-Xlinker", "-rpath,/usr/local/cuda/lib64"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return out_path, [log for _, log in results]


def build(verbose=False, force=False):
    """Compile and link; returns the library path. Skips work when up to date."""
    srcs = [CSRC / s for s in SOURCES] + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + \
        list(INCLUDE.glob("*.h"))
    if LIB.exists() and not force:
        newest = max(p.stat().st_mtime for p in srcs)
        if LIB.stat().st_mtime >= newest:
            return LIB
    BUILD.mkdir(exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if verbose:
        for _, log in results:
            if log:
                print(log)
    tmp = str(LIB) + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-cudart", "shared", "-o", tmp, *[str(o) for o, _ in results],
           "-Xlinker", "-rpath,/usr/local/cuda/lib64"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(verbose="-v" in sys.argv, force=True))
