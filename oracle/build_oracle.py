"""Build recipe for the oracle libraries under oracle/ (test infrastructure).

* ``oracle/_build/libsepx_oracle.so`` -- the CPU restatement (sepx_oracle.c).
* ``oracle/_ref/libsepref.so`` -- the reference's own host C++ (sinc tables,
  random boundary, source stencil, trace/image helpers, cgstep, operator
  classes) compiled from its sources where they lie, against the SEPlib stub
  headers in ``oracle/ref_stubs/`` plus a C shim (``ref_shim.cpp``) that
  exposes them to ctypes.  Built only where the reference tree is present.

Nothing here is part of the product: only tests/, ``__graft_entry__.smoke()``
and bench.py's CPU-baseline leg load these libraries.
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
ORACLE_SO = BUILD / "libsepx_oracle.so"
REF_SO = REF_OUT / "libsepref.so"
REF_ROOT = Path(os.environ.get("SEPX_REFERENCE_ROOT", "/root/reference"))

# The reference's host files that the shim exercises (Born/*.cpp).
REF_SOURCES = [
    "sinc_bob.cpp", "vel_fd_3d.cpp", "source_func_3d.cpp", "deriv_3d.cpp", "laplac_3d.cpp",
    "map_data_3d.cpp", "cgstep.cpp", "hypercube_float.cpp", "hypercube.cpp", "axis.cpp",
    "float_3d.cpp", "my_operator.cpp", "super_vector.cpp", "fd_prop_3d.cpp", "sreg.cpp",
    "sregf.cpp", "oc_float.cpp", "wavefield_insert_3d.cpp", "param_func.cpp", "lin_solver.cpp",
    "combo_oper.cpp", "i_op.cpp", "rtm_zero_op_3d.cpp", "data_rtm_3d.cpp", "image_rtm_3d.cpp",
    "tmute.cpp",
]


# Operator methods that are declared bool but fall off their end without a
# return (Born/deriv_3d.cpp:23,:46, laplac_3d.cpp:44,:96, map_data_3d.cpp:56,:76,
# tmute.cpp:41,:75).  Modern g++ treats that as unreachable and the code runs
# into the next function, so these files are compiled from their text with
# `return true;` inserted before each such closing brace (piped to g++, no
# copy on disk).  Nothing else in the reference text is changed.
PATCH_RETURNS = {"deriv_3d.cpp", "laplac_3d.cpp", "map_data_3d.cpp", "tmute.cpp"}


def _patched_text(src: Path, flags: list[str]) -> bytes:
    probe = subprocess.run([f for f in flags if f != "-w"] + ["-fsyntax-only", "-Wreturn-type", str(src)],
                           capture_output=True, text=True)
    lines = src.read_text().splitlines(keepends=True)
    key = f"{src.name}:"
    for ln in probe.stderr.splitlines():
        if "no return statement" in ln and key in ln:
            row = int(ln.split(key, 1)[1].split(":")[0]) - 1
            lines[row] = lines[row].replace("}", "return true; }", 1)
    return "".join(lines).encode()


def _arch_flags() -> list[str]:
    # fmaf() must compile to the hardware instruction for speed; results are
    # identical either way (fmaf is correctly rounded).
    if platform.machine() in ("x86_64", "AMD64"):
        return ["-mfma"]
    return []


def _newer(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(d.stat().st_mtime <= t for d in deps if d.exists())


def build_oracle(force: bool = False, out: Path | None = None, defines: tuple = ()) -> Path:
    """The oracle library; ``out`` / ``defines`` build a variant elsewhere
    (tests: the stencil block sizes OZB / OYB)."""
    target = ORACLE_SO if out is None else Path(out)
    target.parent.mkdir(parents=True, exist_ok=True)
    deps = [HERE / "sepx_oracle.c", HERE / "sepx_oracle.h", HERE / "sepx_oracle_loops.inc",
            Path(__file__)]
    if not force and not defines and _newer(target, deps):
        return target
    cmd = ["gcc", "-std=gnu11", "-O3", "-fopenmp", "-ffp-contract=off", "-fno-math-errno",
           "-fPIC", "-shared", *_arch_flags(), "-Wall", "-Wno-unused-function",
           *[f"-D{d}" for d in defines],
           str(HERE / "sepx_oracle.c"), "-o", str(target) + ".tmp", "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(str(target) + ".tmp", target)
    return target


def build_ref(force: bool = False) -> Path | None:
    """Compile the reference host code (only where the reference tree exists)."""
    born = REF_ROOT / "Born"
    if not born.is_dir():
        return REF_SO if REF_SO.exists() else None
    REF_OUT.mkdir(exist_ok=True)
    stubs = HERE / "ref_stubs"
    srcs = [born / s for s in REF_SOURCES]
    mine = [stubs / "ref_shim.cpp", stubs / "sep_stubs.cpp", stubs / "ref_gpu_stubs.cpp",
            stubs / "ref_alloc.cpp",
            stubs / "seplib.h", stubs / "sep3d.h", HERE / "sepx_oracle.c", HERE / "sepx_oracle.h",
            HERE / "sepx_oracle_loops.inc"]
    if not force and _newer(REF_SO, srcs + mine + [Path(__file__)]):
        return REF_SO
    objs = []
    common = ["g++", "-std=gnu++11", "-O2", "-fPIC", "-fpermissive", "-w", "-ffp-contract=off",
              "-include", "ctime", "-include", "cmath", "-include", "cstring",
              f"-I{stubs}", f"-I{born}"]
    jobs = []
    for src in srcs + [stubs / "ref_shim.cpp", stubs / "sep_stubs.cpp", stubs / "ref_gpu_stubs.cpp",
                       stubs / "ref_alloc.cpp"]:
        obj = REF_OUT / (src.stem + ".o")
        objs.append(obj)
        if src.name in PATCH_RETURNS:
            text = _patched_text(src, common)
            p = subprocess.Popen(common + ["-x", "c++", "-c", "-", "-o", str(obj)],
                                 stdin=subprocess.PIPE)
            p.stdin.write(text)
            p.stdin.close()
            jobs.append(p)
        else:
            jobs.append(subprocess.Popen(common + ["-c", str(src), "-o", str(obj)]))
    # the oracle loops that stand in for the GPU kernels
    obj = REF_OUT / "sepx_oracle_c.o"
    objs.append(obj)
    jobs.append(subprocess.Popen(["gcc", "-std=gnu11", "-O3", "-fopenmp", "-ffp-contract=off",
                                  "-fno-math-errno", "-fPIC", *_arch_flags(), "-c",
                                  str(HERE / "sepx_oracle.c"), "-o", str(obj)]))
    bad = [j for j in jobs if j.wait() != 0]
    if bad:
        raise RuntimeError("reference host build failed")
    # -Bsymbolic-functions: the zero-tailed new[] of ref_alloc.cpp serves this
    # library's own allocations only
    subprocess.run(["g++", "-shared", "-fopenmp", "-Wl,-Bsymbolic-functions", "-o", str(REF_SO),
                    *map(str, objs), "-lm"], check=True)
    for o in objs:
        o.unlink()
    return REF_SO


REF_CUBIN = REF_OUT / "ref_kernels.cubin"


def build_ref_kernels(force: bool = False) -> Path | None:
    """The reference's own GPU kernels (Born/wave_fkernel.3d8o.cu and the five
    kernels of Born/gpu_funcs_3d.cu) compiled for sm_103a into a cubin, loaded
    by oracle/ref_gpu.py through the driver API on the GPU.  Only device code
    is built, so the cubin needs no host toolchain where it runs.

    Mechanical adjustments to the text handed to nvcc (a temporary file; no
    copy in the repository): the two unused `texture<>` declarations of
    Born/gpu_finite_3d.h:85-86 are dropped (CUDA 12 removed texture
    references); one `__syncthreads()` closes the z loop of wave_kernel and
    wave_kernel_adj (Born/wave_fkernel.3d8o.cu:104, :179: without it a warp
    can overwrite its rows of the shared tile for the next plane while
    another warp still reads them); cuda.h is included for cudaErrors.cu; the
    CUDA 4 SDK helper headers are empty stand-ins (oracle/ref_stubs/cutil_*.h;
    no kernel uses them).  Flags of the reference's Makefile: -ftz=true,
    -maxrregcount=32.  Built only where the reference tree is present."""
    import tempfile
    born = REF_ROOT / "Born"
    if not born.is_dir():
        return REF_CUBIN if REF_CUBIN.exists() else None
    REF_OUT.mkdir(exist_ok=True)
    srcs = [born / "gpu_funcs_3d.cu", born / "gpu_finite_3d.h", born / "wave_fkernel.3d8o.cu",
            born / "cudaErrors.cu", HERE / "ref_stubs" / "cutil_inline.h",
            HERE / "ref_stubs" / "cutil_math.h", Path(__file__)]
    if not force and _newer(REF_CUBIN, srcs):
        return REF_CUBIN
    fin = "".join(ln for ln in (born / "gpu_finite_3d.h").read_text().splitlines(keepends=True)
                  if not ln.lstrip().startswith("texture"))
    wk = (born / "wave_fkernel.3d8o.cu").read_text()
    if wk.count("addr+=stride;") != 2:
        raise RuntimeError("unexpected layout of wave_fkernel.3d8o.cu")
    wk = wk.replace("addr+=stride;", "addr+=stride;\n\t\t__syncthreads();")
    text = (born / "gpu_funcs_3d.cu").read_text()
    text = text.replace('#include "gpu_finite_3d.h"', fin).replace('#include "wave_fkernel.3d8o.cu"', wk)
    text = "#include <cuda.h>\n" + text
    nvcc = str(Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc")
    with tempfile.TemporaryDirectory() as td:
        src = Path(td) / "ref_kernels.cu"
        src.write_text(text)
        tmp = str(REF_CUBIN) + ".tmp"
        subprocess.run([nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-ftz=true",
                        "-maxrregcount=32", "-w", f"-I{HERE / 'ref_stubs'}", f"-I{born}", str(src), "-o",
                        tmp], check=True)
    os.replace(tmp, REF_CUBIN)
    return REF_CUBIN


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
    print(build_ref_kernels(force="--force" in sys.argv))
