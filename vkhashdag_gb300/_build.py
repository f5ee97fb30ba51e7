"""Build recipe of the CUDA extension: nvcc for sm_103a, in-tree.

Compiles every translation unit under csrc/ in parallel and links
libhashdag_gb300.so next to this file.  No CMake.
"""
import concurrent.futures
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libhashdag_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# The read path restates fp32 traversal arithmetic bit for bit: no FMA contraction there.
PER_FILE = {"hd_trace.cu": ["-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"],
            "hd_color.cu": ["-fmad=false", "-prec-div=true", "-ftz=false"]}


def nvcc():
    cand = [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def build(verbose=False, ptxas_info=False):
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    base = [cc, "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
            "-I", os.path.join(HERE, "..", "include")]
    if ptxas_info:
        base += ["-Xptxas", "-v"]

    def one(src):
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = base + PER_FILE.get(src, []) + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        return obj, r.stderr

    with concurrent.futures.ThreadPoolExecutor(max_workers=8) as ex:
        results = list(ex.map(one, sources()))
    objs = [o for o, _ in results]
    if verbose or ptxas_info:
        for _, err in results:
            if err:
                print(err)
    tmp = LIB + ".tmp"
    cmd = [cc, "-shared", *ARCH, "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(verbose=True, ptxas_info="-v" in sys.argv))
