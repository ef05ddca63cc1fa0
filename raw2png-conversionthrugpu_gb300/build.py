"""Build libr2p.so (CUDA kernels + C ABI) in-tree with nvcc for sm_103a.

Translation units compile in parallel into _build/; the shared library lands
next to this file.  Rebuilds only what changed.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libr2p.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

CU_SOURCES = ["k_filter.cu", "k_filter_reg.cu", "k_filter_rows.cu", "k_deflate.cu", "k_lz77.cu", "r2p_engine.cu", "r2p_batch.cu",
              "r2p_server.cu", "r2p_noalloc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-Xcompiler", "-fno-strict-aliasing", "-I" + INCLUDE]


def nvcc():
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, verbose):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if not _stale(obj, [src, __file__] + _headers()):
        return obj
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + ["-c", src, "-o", obj + ".tmp"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    os.replace(obj + ".tmp", obj)
    return obj


# C++17 host layer: the reference's C++ interfaces (gpu_filter.h,
# compression_backend.h, pipeline.h, DicomSource, PngWriter) over the C ABI,
# and the gpu_png_encoder command line.  No CUDA headers: it links libr2p.so.
HOST = os.path.join(HERE, "host")
HOST_LIB = os.path.join(HERE, "libr2p_host.so")
CLI = os.path.join(HERE, "gpu_png_encoder")
HOST_SOURCES = ["gpu_filter.cpp", "compression_backend.cpp", "parallel_deflate.cpp", "png_writer.cpp",
                "file_type.cpp", "dicom_loader.cpp", "image_loader.cpp", "bmp_writer.cpp", "pipeline.cpp",
                "batch_processor.cpp"]
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-Wall", "-Wextra", "-Wno-unused-parameter", "-ffp-contract=off",
             "-I" + os.path.join(HOST, "include"), "-I" + INCLUDE]


def cxx():
    return shutil.which("g++") or "g++"


def _host_headers():
    d = [os.path.join(HOST, "include"), os.path.join(HOST, "src")]
    return [os.path.join(x, f) for x in d for f in os.listdir(x) if f.endswith(".h")] + \
        [os.path.join(INCLUDE, "r2p.h")]


def _compile_host(src, verbose):
    obj = os.path.join(BUILD, "host_" + os.path.basename(src) + ".o")
    if not _stale(obj, [src, __file__] + _host_headers()):
        return obj
    cmd = [cxx()] + CXX_FLAGS + ["-c", src, "-o", obj + ".tmp"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("g++ failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    os.replace(obj + ".tmp", obj)
    return obj


def _link(out, cmd, deps, verbose):
    if not _stale(out, deps):
        return
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link of %s failed:\n%s%s" % (os.path.basename(out), r.stdout, r.stderr))
    os.replace(out + ".tmp", out)


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(CSRC, f) for f in CU_SOURCES]
    hsrcs = [os.path.join(HOST, "src", f) for f in HOST_SOURCES + ["main.cpp"]]
    with cf.ThreadPoolExecutor(max_workers=len(srcs) + len(hsrcs)) as ex:
        fo = [ex.submit(_compile, s, verbose) for s in srcs]
        fh = [ex.submit(_compile_host, s, verbose) for s in hsrcs]
        objs = [f.result() for f in fo]
        hobjs = [f.result() for f in fh]
    _link(LIB, [nvcc()] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lpthread"], objs, verbose)
    rpath = ["-Wl,-rpath,$ORIGIN", "-L" + HERE]
    _link(HOST_LIB, [cxx(), "-shared", "-o", HOST_LIB + ".tmp"] + hobjs[:-1] + rpath + ["-lr2p", "-lpthread"],
          hobjs[:-1] + [LIB], verbose)
    _link(CLI, [cxx(), "-o", CLI + ".tmp", hobjs[-1]] + rpath + ["-lr2p_host", "-lr2p", "-lpthread"],
          [hobjs[-1], HOST_LIB, LIB], verbose)
    return LIB


if __name__ == "__main__":
    print(build("-v" in sys.argv))
