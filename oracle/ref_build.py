"""Build recipe for the reference oracle (test infrastructure): breseq's own sources, unmodified and
read in place from the reference tree, compiled with g++ against the clean-room htslib subset and the
miniz and config.h stand-ins in oracle/refbuild/, plus the driver oracle/refbuild/harness.cpp.

Output: oracle/_ref/ref_harness (git-ignored).  Needs the reference tree (BRESEQ_REF_SRC or
/root/reference/src/breseq) and zlib; where the tree is absent (the GPU machine) build() returns None and
the tests that use the binary skip.  The reference's own build system (autotools) is not used.

    python oracle/ref_build.py [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SHIM = os.path.join(HERE, "refbuild")
OUT = os.path.join(HERE, "_ref")
BIN = os.path.join(OUT, "ref_harness")
# command-line programs of the reference (they hold main()); everything else is its library, but
# coverage_distribution.cpp is compiled inside refbuild/covfit.cpp instead (its fit is file-local)
MAINS = {"breseq_cmdline.cpp", "gdtools_cmdline.cpp", "coverage_table_cmdline.cpp"}
INCLUDED = {"coverage_distribution.cpp"}


def ref_src() -> str | None:
    d = os.environ.get("BRESEQ_REF_SRC", "/root/reference/src/breseq")
    return d if os.path.isfile(os.path.join(d, "identify_mutations.cpp")) else None


def data_path() -> str | None:
    src = ref_src()
    return os.path.normpath(os.path.join(src, "..", "share", "breseq")) if src else None


def build(force: bool = False) -> str | None:
    src = ref_src()
    if src is None:
        return None
    srcs = sorted(f for f in os.listdir(src) if f.endswith(".cpp") and f not in MAINS and f not in INCLUDED)
    ours = [os.path.join(SHIM, f) for f in ("hts_shim.cpp", "harness.cpp", "covfit.cpp")]
    deps = [os.path.join(src, f) for f in os.listdir(src)] + ours
    for root, _, files in os.walk(os.path.join(SHIM, "include")):
        deps += [os.path.join(root, f) for f in files]
    if not force and os.path.exists(BIN) and os.path.getmtime(BIN) >= max(os.path.getmtime(d) for d in deps):
        return BIN
    obj_dir = os.path.join(OUT, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    # DATADIR relative: the harness points the data path at the tree's share/breseq (BRESEQ_DATA_PATH)
    flags = ["-std=c++11", "-O2", "-w", "-I", os.path.join(SHIM, "include"), "-I", src, '-DDATADIR="../share/breseq/"']

    def cc(path):
        obj = os.path.join(obj_dir, os.path.basename(path)[:-4] + ".o")
        r = subprocess.run(["g++"] + flags + ["-c", path, "-o", obj], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"g++ failed on {path}:\n{r.stderr[-4000:]}")
        return obj

    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        lib_objs = list(ex.map(cc, [os.path.join(src, f) for f in srcs]))
        shim_obj, harness_obj, covfit_obj = list(ex.map(cc, ours))
    archive = os.path.join(obj_dir, "libbreseq_ref.a")
    if os.path.exists(archive):
        os.remove(archive)
    subprocess.check_call(["ar", "rcs", archive] + lib_objs)
    subprocess.check_call(["g++", "-o", BIN + ".tmp", harness_obj, covfit_obj, archive, shim_obj, "-lz", "-lpthread"])
    os.replace(BIN + ".tmp", BIN)
    return BIN


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
