"""Build libmolgpu.so (sm_103a) in-tree: ``python methodoflines.jl_gb300/build.py``.

Each CUDA translation unit is compiled in parallel with nvcc, then linked into
``methodoflines.jl_gb300/molgpu/_lib/libmolgpu.so``.  No cmake, no torch
extension machinery: the library is plain C ABI over the CUDA runtime.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "molgpu", "_lib")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libmolgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the molgpu CUDA library cannot be built")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(BUILD_DIR, "mol_embedded.inc"))
    deps.append(os.path.join(ROOT, "include", "molgpu.h"))
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


EMBED = ["molgpu.h", "mol_device.cuh", "mol_vjp.cuh", "mol_kernels.cuh"]


def _embed() -> None:
    """Write the device headers as C string literals: NVRTC compiles the generated code against them."""
    texts = []
    for name in EMBED:
        path = os.path.join(ROOT, "include", name) if name == "molgpu.h" else os.path.join(CSRC, name)
        txt = open(path).read()
        if ")MOLRAW\"" in txt:
            raise RuntimeError("raw-string delimiter found in " + name)
        texts.append(txt)
    body = "static const char* const kEmbedNames[] = {" + ", ".join('"%s"' % n for n in EMBED) + "};\n"
    body += "static const char* const kEmbedTexts[] = {\n" + ",\n".join('R"MOLRAW(' + t + ')MOLRAW"' for t in texts)
    body += "};\n"
    out = os.path.join(BUILD_DIR, "mol_embedded.inc")
    if not os.path.exists(out) or open(out).read() != body:
        with open(out, "w") as fh:
            fh.write(body)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(BUILD_DIR, exist_ok=True)
    _embed()
    cc = nvcc()
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + os.path.join(ROOT, "include"),
                     "-I" + CSRC, "-I" + BUILD_DIR]
    objs = []
    jobs = []
    for src in sources():
        obj = os.path.join(BUILD_DIR, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, src):
            jobs.append([cc] + common + ["-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose:
            print(" ".join(cmd))
        return r

    if jobs:
        with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
            list(ex.map(run, jobs))
    if force or jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        run([cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-ldl"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
