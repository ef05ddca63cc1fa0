"""Build recipe for the oracle (test infrastructure, never shipped).

Outputs:
  oracle/liboracle.so  -- oracle.c (window/filter/unfilter restatement) plus
                          port_cpu.cpp (CPU restatement of the reference's
                          strip-parallel zlib encode path), linked against zlib.
  oracle/_ref/...      -- built only where the reference tree is present, from
                          the reference's own sources, left where they lie:
     libref_window.so   src/batch_processor.cpp via ref_window_harness.cpp
     ref_bmp_runner     src/pipeline.cpp + src/bmp_writer.cpp via ref_bmp_harness.cpp
     libref_cpu.so      src/parallel_deflate.cpp + src/png_writer.cpp via
                        ref_cpu_harness.cpp
     gpu_filter_ref_fastmath.cubin / gpu_filter_ref_ieee.cubin
                        src/gpu_filter.cu for sm_103a, once with the
                        reference's own --use_fast_math and once with IEEE
                        division and no FMA contraction.
oracle/_ref is git-ignored.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference tree: R2P_REFERENCE_DIR, or --reference DIR on the command
# line, else the location this build's container mounts it at
REF = os.environ.get("R2P_REFERENCE_DIR", "/root/reference")
REF_DIR = os.path.join(HERE, "_ref")


def _newer(out, srcs):
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(s) <= t for s in srcs if os.path.exists(s))


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def build_oracle(verbose=False):
    out = os.path.join(HERE, "liboracle.so")
    srcs = [os.path.join(HERE, f) for f in ("oracle.c", "port_cpu.cpp", "build_oracle.py")]
    if _newer(out, srcs):
        return out
    tmp = out + ".tmp"
    flags = ["-O2", "-ffp-contract=off", "-fPIC", "-fno-strict-aliasing"]
    obj_c = os.path.join(HERE, "_oracle_c.o")
    _run(["gcc", "-std=c11"] + flags + ["-c", os.path.join(HERE, "oracle.c"), "-o", obj_c], verbose)
    _run(["g++", "-std=c++17"] + flags + ["-shared", obj_c, os.path.join(HERE, "port_cpu.cpp"),
                                          "-o", tmp, "-lz", "-lpthread"], verbose)
    os.remove(obj_c)
    os.replace(tmp, out)
    return out


def build_ref(verbose=False):
    """Compile the reference's own sources (only where they are present)."""
    if not os.path.isdir(os.path.join(REF, "src")):
        return False
    os.makedirs(REF_DIR, exist_ok=True)
    shim = os.path.join(REF_DIR, "shim")
    os.makedirs(shim, exist_ok=True)
    # The reference includes the MSVC-only <intrin.h> for _mm_prefetch; a
    # portable stand-in maps it to the GCC prefetch builtin.
    with open(os.path.join(shim, "intrin.h"), "w") as f:
        f.write("#pragma once\n#define _MM_HINT_T0 0\n"
                "#define _mm_prefetch(p, h) __builtin_prefetch((const void*)(p))\n")
    inc = ["-I" + os.path.join(REF, "src"), "-I" + os.path.join(REF, "include"), "-I" + shim]
    flags = ["-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-w"]
    win = os.path.join(REF_DIR, "libref_window.so")
    if not _newer(win, [os.path.join(HERE, "ref_window_harness.cpp")]):
        _run(["g++"] + flags + inc + [os.path.join(HERE, "ref_window_harness.cpp"), "-o", win,
                                      "-lpthread"], verbose)
    cpu = os.path.join(REF_DIR, "libref_cpu.so")
    if not _newer(cpu, [os.path.join(HERE, "ref_cpu_harness.cpp")]):
        _run(["g++"] + flags + inc + [os.path.join(HERE, "ref_cpu_harness.cpp"),
                                      os.path.join(REF, "src", "parallel_deflate.cpp"),
                                      os.path.join(REF, "src", "png_writer.cpp"),
                                      "-o", cpu, "-lz", "-lpthread"], verbose)
    # the reference's BMP export: src/pipeline.cpp + src/bmp_writer.cpp run by
    # a small executable (unresolved GPU/decoder symbols are never reached)
    bmp = os.path.join(REF_DIR, "ref_bmp_runner")
    if not _newer(bmp, [os.path.join(HERE, "ref_bmp_harness.cpp")]):
        _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-w"] + inc +
             [os.path.join(HERE, "ref_bmp_harness.cpp"), "-o", bmp,
              "-Wl,--unresolved-symbols=ignore-all", "-lpthread"], verbose)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cu = os.path.join(REF, "src", "gpu_filter.cu")
    for tag, extra in (("fastmath", ["--use_fast_math"]),
                       ("ieee", ["-prec-div=true", "-prec-sqrt=true", "-fmad=false"])):
        cub = os.path.join(REF_DIR, "gpu_filter_ref_%s.cubin" % tag)
        if not os.path.exists(cub):
            _run([nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
                  "-I" + os.path.join(REF, "include"), cu, "-o", cub] + extra, verbose)
    return True


def build_ref_gpu_runner(verbose=False):
    """oracle/_ref/libref_gpu_runner.so: a driver-API launcher for the
    reference kernels in the cubins build_ref() made (on a machine with a
    GPU driver; needs only the CUDA headers and the driver stub to build)."""
    out = os.path.join(REF_DIR, "libref_gpu_runner.so")
    src = os.path.join(HERE, "ref_gpu_runner.cpp")
    if _newer(out, [src]):
        return out
    os.makedirs(REF_DIR, exist_ok=True)
    cuda = os.path.dirname(os.path.dirname(shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"))
    _run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", src, "-I" + os.path.join(cuda, "include"),
          "-L" + os.path.join(cuda, "lib64", "stubs"), "-L" + os.path.join(cuda, "lib64"), "-lcuda", "-o", out],
         verbose)
    return out


if __name__ == "__main__":
    v = "-v" in sys.argv
    if "--reference" in sys.argv:
        REF = sys.argv[sys.argv.index("--reference") + 1]
    print(build_oracle(v))
    print("reference harness built:", build_ref(v))
