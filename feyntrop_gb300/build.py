"""Builds the native library and the `feyntrop` command in-tree.

    python -m feyntrop_gb300.build        (or feyntrop_gb300.build.build())

Outputs (git-ignored) in feyntrop_gb300/_build/:
    libfeyntrop_gb300.so   C ABI of include/feyntrop_gb300.h: host preprocessing, the
                           runtime compiler driver for the per-topology sampling kernels,
                           and the ahead-of-time sm_103a kernels (csrc/kernels/aot.cu)
    feyntrop               the reference's CLI contract on top of the library

The sampling kernels themselves are compiled per graph topology at run time
(csrc/jit.cpp); `precompile()` compiles a list of topologies ahead of use.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
CXX = os.environ.get("CXX", "g++")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

SOURCES = ["json.cpp", "problem.cpp", "xoshiro.cpp", "jit.cpp", "runtime.cpp", "batch.cpp", "tune.cpp", "driver.cpp"]
LIB = os.path.join(OUT, "libfeyntrop_gb300.so")
CLI = os.path.join(OUT, "feyntrop")


def _embed():
    src = os.path.join(CSRC, "kernels", "sample_body.cuh")
    dst = os.path.join(OUT, "sample_body_embed.cpp")
    text = open(src).read()
    chunks = [text[i:i + 8000] for i in range(0, len(text), 8000)]
    body = "\n".join('R"FTBODY(%s)FTBODY"' % c for c in chunks)
    code = ("// generated by feyntrop_gb300/build.py from csrc/kernels/sample_body.cuh\n"
            "extern const char* ft_sample_body_source;\nconst char* ft_sample_body_source =\n%s;\n" % body)
    if not os.path.exists(dst) or open(dst).read() != code:
        with open(dst, "w") as f:
            f.write(code)
    return dst


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s%s" % (" ".join(cmd), p.stdout, p.stderr))
    return p


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".hpp")]
    headers += [os.path.join(REPO, "include", "feyntrop_gb300.h"), os.path.join(CSRC, "kernels", "aot.hpp")]
    embed = _embed()
    jobs = []
    objs = []
    cflags = ["-std=c++17", "-O2", "-fPIC", "-Wall", "-Wno-unused-function", "-I" + os.path.join(CUDA, "include")]
    for s in SOURCES + [embed]:
        path = s if os.path.isabs(s) else os.path.join(CSRC, s)
        obj = os.path.join(OUT, os.path.basename(path).replace(".cpp", ".o"))
        objs.append(obj)
        if _stale(obj, [path] + headers):
            jobs.append([CXX] + cflags + ["-c", path, "-o", obj])
    aot_src = os.path.join(CSRC, "kernels", "aot.cu")
    aot_obj = os.path.join(OUT, "aot.o")
    objs.append(aot_obj)
    if _stale(aot_obj, [aot_src] + headers):
        jobs.append([NVCC] + ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-c", aot_src,
                                     "-o", aot_obj])
    cli_obj = os.path.join(OUT, "cli.o")
    if _stale(cli_obj, [os.path.join(CSRC, "cli.cpp")] + headers):
        jobs.append([CXX] + cflags + ["-c", os.path.join(CSRC, "cli.cpp"), "-o", cli_obj])
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        for r in ex.map(_run, jobs):
            if verbose and r.stderr:
                sys.stderr.write(r.stderr)
    libs = ["-L" + os.path.join(CUDA, "lib64"), "-lcudart", "-lnvrtc", "-lpthread", "-ldl",
            "-Wl,-rpath," + os.path.join(CUDA, "lib64")]
    if _stale(LIB, objs):
        _run([CXX, "-shared", "-o", LIB] + objs + libs)
    if _stale(CLI, [cli_obj, LIB]):
        _run([CXX, "-o", CLI, cli_obj, "-L" + OUT, "-lfeyntrop_gb300", "-Wl,-rpath,$ORIGIN"] + libs)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    print(LIB)
