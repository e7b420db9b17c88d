"""In-tree build of libgpis_gb300.so for sm_103a (nvcc, no cmake).

Translation units compile in parallel with -gencode arch=compute_103a,code=sm_103a;
the -Xptxas -v report of the device code goes to _build/ptxas.log.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libgpis_gb300.so")
ROOT = os.path.dirname(HERE)

SOURCES = ["flights.cu", "gpis_abi.cu", "gpis_static.cu", "render.cu", "backend.cu", "proposal.cu",
           "medium_json.cpp", "medium_adapter.cpp"]
# per-file flags: the path tracer rounds every float expression as its CPU restatement
EXTRA = {"render.cu": ["-fmad=false"]}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(ROOT, "include", "gpis.h"))
    files.append(os.path.abspath(__file__))
    return files


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    common = ["-std=c++17", "-O3", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include")]

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc, *ARCH, *common, *EXTRA.get(src, []), "-lineinfo", "-Xptxas", "-v", "-c",
               os.path.join(CSRC, src), "-o", obj]
        if src.endswith(".cpp"):
            cmd = [nvcc, *common, "-x", "c++", "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return obj, r.stderr

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    with open(os.path.join(BUILD, "ptxas.log"), "w") as f:
        for (_, log), src in zip(results, SOURCES):
            f.write(f"== {src}\n{log}\n")
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-cudart=static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
