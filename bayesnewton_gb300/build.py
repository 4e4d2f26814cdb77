"""Build libbnx.so for sm_103a: one translation unit per compiled configuration,
compiled in parallel with nvcc, linked into bayesnewton_gb300/libbnx.so."""
import concurrent.futures as cf
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libbnx.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def configs():
    """(dtype, P, blocks) triples listed in bn_layout.h."""
    text = open(os.path.join(CSRC, "bn_layout.h")).read()
    out = []
    for t, p, blocks in re.findall(r"X\((float|double), (\d), ([\d, ]+)\)", text):
        out.append((t, int(p), tuple(int(b) for b in blocks.split(","))))
    return out


def _sources():
    os.makedirs(BUILD, exist_ok=True)
    units = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))
    for t, p, blocks in configs():
        name = "inst_%s_p%d_%s.cu" % (t, p, "_".join(map(str, blocks)))
        path = os.path.join(BUILD, name)
        body = ('#include "%s"\nnamespace bn {\ntemplate EngineBase* make_engine<%s, Layout<%s>, %d>'
                '(int64_t, int, int, bool, int*);\n}\n') % (
            os.path.join(CSRC, "bn_engine.cuh"), t, ", ".join(map(str, blocks)), p)
        if not os.path.exists(path) or open(path).read() != body:
            with open(path, "w") as f:
                f.write(body)
        units.append(path)
    return units


def _compile(src, deps_mtime, verbose):
    obj = os.path.join(BUILD, os.path.basename(src).replace(".cu", ".o"))
    if os.path.exists(obj) and os.path.getmtime(obj) > max(deps_mtime, os.path.getmtime(src)):
        return obj
    cmd = [nvcc()] + ARCH + FLAGS + ["-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s" % (src, r.stderr[-4000:]))
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


def build(jobs=None, verbose=False):
    srcs = _sources()
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(HERE, "..", "include", "bnx.h")]
    deps = max(os.path.getmtime(h) for h in hdrs)
    jobs = jobs or max(1, os.cpu_count() or 1)
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, deps, verbose), srcs))
    if os.path.exists(LIB) and os.path.getmtime(LIB) > max(os.path.getmtime(o) for o in objs):
        return LIB
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stderr[-4000:])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
