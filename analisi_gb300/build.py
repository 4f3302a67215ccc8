"""In-tree build of the analisi_gb300 native libraries.

    python -m analisi_gb300.build          # or __graft_entry__.build()

Produces, under analisi_gb300/_build/:
  libgofr_gb300.so   the CUDA engine and its C ABI (include/gofr_gb300.h),
                     compiled for sm_103a only
  pyanalisi*.so      the pybind11 module with the reference's Gofrt /
                     Trajectory / BoxFormat API, linked against libgofr_gb300
  analisi            the command-line front end (-g/-F options)
and, on request (build_engine(debug_bounds=True)), analisi_gb300/_build_debug/
libgofr_gb300.so with the GOFR_DEBUG_BOUNDS device-side index checks.

Translation units are compiled in parallel; nothing here needs cmake.
Host code is compiled with -ffp-contract=off so that the host-side bin
thresholds use the same separate IEEE operations as the reference.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
OUT = os.path.join(HERE, "_build")
OUT_DEBUG = os.path.join(HERE, "_build_debug")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math", "-Xptxas", "-v"]
CU_SOURCES = ["gofr_kernels.cu", "gofr_cells.cu", "gofr_cellw.cu", "gofr_capi.cu", "gofr_peaks.cu",
              "gofr_noalloc.cu", "gofr_msd.cu", "gofr_neigh.cu", "gofr_norm.cu"]
LIB_NAME = "libgofr_gb300.so"


def nvcc():
    """nvcc from PATH, else from the CUDA toolkit that $CUDA_HOME / $CUDA_PATH
    name, else from the toolkit PyTorch was told about (its own lookup)."""
    cand = shutil.which("nvcc")
    if cand:
        return cand
    homes = [os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH")]
    try:
        from torch.utils import cpp_extension
        homes.append(cpp_extension.CUDA_HOME)
    except Exception:  # torch absent or without CUDA: only the first two
        pass
    for h in homes:
        if h and os.path.exists(os.path.join(h, "bin", "nvcc")):
            return os.path.join(h, "bin", "nvcc")
    raise RuntimeError("nvcc not found: put it on PATH or set CUDA_HOME")


def _run(cmd, log=None):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if log is not None:
        with open(log, "w") as f:
            f.write(" ".join(cmd) + "\n" + p.stdout)
    if p.returncode != 0:
        sys.stderr.write(p.stdout)
        raise RuntimeError("command failed: " + " ".join(cmd))
    return p.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _deps_cuda():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    return files + [os.path.join(INCLUDE, "gofr_gb300.h")]


def build_engine(force=False, jobs=None, debug_bounds=False):
    """Compile the CUDA engine into analisi_gb300/_build/libgofr_gb300.so, or
    with debug_bounds the GOFR_DEBUG_BOUNDS variant (device-side index checks
    that set an error word) into analisi_gb300/_build_debug/."""
    out = OUT_DEBUG if debug_bounds else OUT
    os.makedirs(out, exist_ok=True)
    lib = os.path.join(out, LIB_NAME)
    deps = _deps_cuda()
    if not force and not _stale(lib, deps):
        return lib
    nv = nvcc()
    extra = ["-DGOFR_DEBUG_BOUNDS"] if debug_bounds else []
    objs = []
    cmds = []
    for src in CU_SOURCES:
        obj = os.path.join(out, src.replace(".cu", ".o"))
        objs.append(obj)
        cmds.append(([nv] + ARCH + NVCC_FLAGS + extra + ["-I", INCLUDE, "-I", CSRC, "-c",
                      os.path.join(CSRC, src), "-o", obj],
                     os.path.join(out, src.replace(".cu", ".ptxas.log"))))
    with cf.ThreadPoolExecutor(max_workers=jobs or len(cmds)) as ex:
        list(ex.map(lambda c: _run(*c), cmds))
    _run([nv] + ARCH + ["-shared", "-o", lib + ".tmp"] + objs)
    os.replace(lib + ".tmp", lib)
    return lib


def _pybind_include():
    try:
        import pybind11  # noqa: F401
        return pybind11.get_include()
    except ImportError:
        # PyTorch ships the pybind11 headers; only the headers are used.
        import importlib.util
        spec = importlib.util.find_spec("torch")
        if spec is None or not spec.submodule_search_locations:
            raise RuntimeError("pybind11 headers not found (neither pybind11 nor torch)")
        return os.path.join(list(spec.submodule_search_locations)[0], "include")


def build_host(force=False):
    """Compile the pybind11 module and the CLI against libgofr_gb300.so."""
    lib = build_engine()
    cxx = os.environ.get("CXX", "g++")
    suffix = sysconfig.get_config_var("EXT_SUFFIX")
    mod = os.path.join(OUT, "pyanalisi" + suffix)
    cli = os.path.join(OUT, "analisi")
    host_srcs = [os.path.join(HOST, f) for f in os.listdir(HOST)]
    common = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
              "-I", INCLUDE, "-I", HOST]
    link = ["-L", OUT, "-lgofr_gb300", "-Wl,-rpath,$ORIGIN", "-lpthread"]
    jobs = []
    if os.path.exists(os.path.join(HOST, "pyanalisi.cpp")) and (
            force or _stale(mod, host_srcs + [lib])):
        jobs.append([cxx] + common + ["-shared", "-I", _pybind_include(),
                     "-I", sysconfig.get_paths()["include"],
                     os.path.join(HOST, "pyanalisi.cpp"), os.path.join(HOST, "trajectory.cpp"),
                     os.path.join(HOST, "lammps_file.cpp"), "-o", mod] + link)
    if os.path.exists(os.path.join(HOST, "analisi_main.cpp")) and os.path.exists(
            os.path.join(HOST, "lammps_file.cpp")) and (
            force or _stale(cli, host_srcs + [lib])):
        jobs.append([cxx] + common + [os.path.join(HOST, "analisi_main.cpp"),
                     os.path.join(HOST, "trajectory.cpp"), os.path.join(HOST, "lammps_file.cpp"),
                     "-o", cli] + link)
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    return mod, cli


def build_all(force=False):
    lib = build_engine(force=force)
    mod, cli = build_host(force=force)
    return lib, mod, cli


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv))
