"""Build the real SEAL-4.1-bs library from the NEXUS sources -- TEST INFRASTRUCTURE.

Compiles thirdparty/SEAL-4.1-bs/native/src/seal/**.{cpp,c} where they lie in
the NEXUS tree with g++/gcc directly (SEAL's own CMake build is not used) plus
oracle/seal_shim.cpp, and links oracle/_ref/libseal_shim.so.  The one header
SEAL's CMake would generate, seal/util/config.h, is written by this recipe from
config.h.in with the options below (HEXL, MSGSL, zlib and zstd off; they
cannot be fetched offline).  Nothing from the NEXUS tree is copied into the
repository; all outputs go to oracle/_ref/ (git-ignored).

The NEXUS sources exist only on the development machine, so the library is
built there; tests that need it skip when it is absent.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import re
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
NEXUS_TREE = Path(os.environ.get("NEXUS_REFERENCE", "/root/reference"))
SEAL_SRC = NEXUS_TREE / "thirdparty" / "SEAL-4.1-bs" / "native" / "src"
LIB = OUT / "libseal_shim.so"
# NEXUS's operators on SEAL (src/ in the NEXUS tree).  src/ckks_evaluator.cpp
# names compr_mode_type::zstd (a deprecated helper); zstd is compiled out of
# SEAL here, so that one enumerator is mapped to `none` with -Dzstd=none.
NEXUS_SRC = NEXUS_TREE / "src"
NEXUS_OPS = ["ckks_evaluator.cpp", "gelu.cpp", "softmax.cpp", "layer_norm.cpp", "matrix_mul.cpp"]

CONFIG_ON = ["SEAL_USE_STD_BYTE", "SEAL_USE_SHARED_MUTEX", "SEAL_USE_IF_CONSTEXPR", "SEAL_USE_MAYBE_UNUSED",
             "SEAL_USE_NODISCARD", "SEAL_USE_STD_FOR_EACH_N", "SEAL_USE_INTRIN", "SEAL_USE___INT128",
             "SEAL_USE___BUILTIN_CLZLL"]


def reference_available() -> bool:
    return (SEAL_SRC / "seal" / "evaluator.cpp").exists()


def _write_config():
    tmpl = (SEAL_SRC / "seal" / "util" / "config.h.in").read_text()
    cfg = tmpl.replace("@SEAL_VERSION@", "4.1.2").replace("@SEAL_VERSION_MAJOR@", "4")
    cfg = cfg.replace("@SEAL_VERSION_MINOR@", "1").replace("@SEAL_VERSION_PATCH@", "2")

    def repl(m):
        name = m.group(1)
        if name == "SEAL_DEFAULT_PRNG":
            return "#define SEAL_DEFAULT_PRNG Blake2xb"
        return f"#define {name}" if name in CONFIG_ON else f"/* #undef {name} */"

    cfg = re.sub(r"#cmakedefine (\w+)[^\n]*", repl, cfg)
    d = OUT / "include" / "seal" / "util"
    d.mkdir(parents=True, exist_ok=True)
    p = d / "config.h"
    if not p.exists() or p.read_text() != cfg:
        p.write_text(cfg)


def build(jobs: int | None = None) -> Path:
    if not reference_available():
        raise FileNotFoundError(f"SEAL sources not found under {SEAL_SRC}")
    OUT.mkdir(exist_ok=True)
    _write_config()
    objdir = OUT / "obj"
    objdir.mkdir(exist_ok=True)
    srcs = sorted((SEAL_SRC / "seal").glob("*.cpp")) + sorted((SEAL_SRC / "seal" / "util").glob("*.cpp")) + \
        sorted((SEAL_SRC / "seal" / "util").glob("*.c")) + [NEXUS_SRC / f for f in NEXUS_OPS] + \
        [HERE / "seal_shim.cpp"]
    inc = ["-I", str(OUT / "include"), "-I", str(SEAL_SRC), "-I", str(NEXUS_SRC)]
    todo, objs = [], []
    for s in srcs:
        o = objdir / (s.parent.name + "_" + s.name + ".o")
        if s.parent == NEXUS_SRC:
            o = objdir / ("nexus_" + s.name + ".o")
        objs.append(o)
        if not o.exists() or o.stat().st_mtime < s.stat().st_mtime:
            todo.append((s, o))

    def cc(item):
        s, o = item
        if s.suffix == ".c":
            cmd = ["gcc", "-O2", "-fPIC", "-std=c11"] + inc + ["-c", str(s), "-o", str(o)]
        else:
            cmd = ["g++", "-O2", "-fPIC", "-std=c++17", "-ffp-contract=off"] + inc + ["-c", str(s), "-o", str(o)]
            if s.parent == NEXUS_SRC:
                cmd.insert(1, "-Dzstd=none")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"compile failed: {s}\n{r.stderr[-4000:]}")

    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as ex:
            list(ex.map(cc, todo))
    if todo or not LIB.exists():
        r = subprocess.run(["g++", "-shared", "-o", str(LIB)] + [str(o) for o in objs] + ["-lpthread"],
                           capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError("link failed:\n" + r.stderr[-4000:])
    return LIB


if __name__ == "__main__":
    print(build())
