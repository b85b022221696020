"""Builds libralgpu.so in-tree (blazingdb-ral_gb300/_build/).

Host C++ with g++, ahead-of-time kernels with nvcc for sm_103a only, linked
with the static CUDA runtime and NVRTC.  device_rt.cuh is embedded as a string
so that the JIT needs no include path at run time.  Rebuilds only what
changed; translation units compile in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libralgpu.so")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")

CPP = ["program.cpp", "frontend.cpp", "codegen.cpp", "jit.cpp", "engine.cpp", "filter.cpp", "batch.cpp", "server.cpp",
       "selftest.cpp", "aggregate.cpp", "category.cpp", "textscan.cpp", "parquet_meta.cpp", "parquet_scan.cpp", "capi.cpp"]
CU = ["kernels.cu", "noalloc.cu"]
HEADERS = ["program.h", "frontend.h", "codegen.h", "jit.h", "engine.h", "filter.h", "batch.h", "server.h", "kernels.h", "device_rt.cuh", "softfp.cuh",
           "textscan.cuh", "textscan.h", "parquet_meta.h"]
INCLUDES = [f"-I{os.path.join(ROOT, 'include')}", f"-I{CSRC}", f"-I{os.path.join(CUDA, 'include')}"]
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _mtime(p: str) -> float:
    return os.path.getmtime(p) if os.path.exists(p) else 0.0


def _deps_mtime() -> float:
    hs = [os.path.join(CSRC, h) for h in HEADERS]
    hs += [os.path.join(ROOT, "include", "ral", f) for f in os.listdir(os.path.join(ROOT, "include", "ral"))]
    return max(_mtime(h) for h in hs)


def _embed_prelude() -> str:
    # softfp.cuh first: device_rt.cuh then skips its #include of it (NVRTC has no include path)
    src = open(os.path.join(CSRC, "softfp.cuh")).read() + "\n" + open(os.path.join(CSRC, "device_rt.cuh")).read()
    out = os.path.join(OUT, "prelude_embed.cpp")
    scan = open(os.path.join(CSRC, "textscan.cuh")).read()
    text = ('// generated from csrc/softfp.cuh, csrc/device_rt.cuh and csrc/textscan.cuh by build.py\n'
            'extern "C" const char* const ral_prelude_source;\n'
            'extern "C" const char* const ral_prelude_source = R"RALPRELUDE(' + src + ')RALPRELUDE";\n'
            '// the field parsers of the text scan kernels (prepended to their generated source)\n'
            'extern "C" const char* const ral_textscan_source;\n'
            'extern "C" const char* const ral_textscan_source = R"RALPRELUDE(' + scan + ')RALPRELUDE";\n')
    if not os.path.exists(out) or open(out).read() != text:
        with open(out, "w") as f:
            f.write(text)
    return out


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    prelude = _embed_prelude()
    deps = _deps_mtime()
    jobs = []
    objs = []
    for src in CPP + [prelude]:
        path = src if os.path.isabs(src) else os.path.join(CSRC, src)
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _mtime(obj) < max(_mtime(path), deps):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function", *INCLUDES,
                         "-c", path, "-o", obj])
    for src in CU:
        path = os.path.join(CSRC, src)
        obj = os.path.join(OUT, src + ".o")
        objs.append(obj)
        if force or _mtime(obj) < max(_mtime(path), deps):
            jobs.append([NVCC, *GENCODE, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", *INCLUDES,
                         "-c", path, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
            for out in ex.map(_run, jobs):
                if verbose and out.strip():
                    print(out)
    if force or jobs or _mtime(LIB) < max(_mtime(o) for o in objs):
        tmp = LIB + ".tmp"
        _run([NVCC, *GENCODE, "-shared", "-o", tmp, *objs, f"-L{os.path.join(CUDA, 'lib64')}", "-lnvrtc", "-lnvJitLink",
              "-Xlinker", f"-rpath,{os.path.join(CUDA, 'lib64')}"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
