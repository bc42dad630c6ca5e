"""Builds the reference's own solver into oracle/_ref (the recipe).

TEST INFRASTRUCTURE ONLY.  Compiles the reference's sources where they lie
(NikitaMatckevich/SWE_FVM: src/*.cpp with include/*.h) with g++, against the
hand-written Eigen subset in oracle/eigen_subset (Eigen itself is fetched over
the network by the reference's CMakeLists.txt:14-19 and is absent here), plus
the C driver oracle/ref/ref_driver.cpp, into:

  oracle/_ref/libswe_ref.so        Q1 and Q20 patched (the parity target)
  oracle/_ref/libswe_ref_q20lit.so Q1 patched only: the positivity test of
                                   src/MUSCLObject.cpp:68 as Eigen's release
                                   build evaluates it (see below)

Nothing is copied into the repository.  Two files get a one-line edit, applied
to copies written under oracle/_ref/patched (git-ignored build output):

  Q1  src/Bathymetry.cpp:29-31  Domain::E(e) returns an uninitialised Point{};
      it becomes the midpoint of the edge's two nodes, (P0 + P1) * 0.5, the
      reading the restatement and the device code use.
  Q20 src/MUSCLObject.cpp:68    `hp = wp - b.P(ip)` subtracts a 3 x 3 block
      from a 3-vector.  Eigen asserts on it in debug builds; a release build
      reads column 0 of the block, i.e. subtracts node ip[0]'s (x, y, z) from
      the three vertex levels.  The evident intent, vertex level minus that
      vertex's bathymetry, is `wp - b.P(ip).row(2).transpose()`.

Both builds force-include oracle/ref/prelude.h (the Q18 reading of the
unqualified abs and the correctly rounded cube root shared with the
restatement) and use -O3 -DNDEBUG -ffp-contract=off: the reference's release
flags (CMakeLists.txt:6) without floating-point contraction, so results do
not depend on whether the host compiler fuses multiply-adds.

Usage: python oracle/ref/build_ref.py [reference root]
       (default: $SWE_REFERENCE_ROOT, else /root/reference)
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
LIB = os.path.join(OUT, "libswe_ref.so")
LIB_Q20LIT = os.path.join(OUT, "libswe_ref_q20lit.so")
EIGEN = os.path.join(ORACLE, "eigen_subset")
PRELUDE = os.path.join(HERE, "prelude.h")
DRIVER = os.path.join(HERE, "ref_driver.cpp")
RESTATEMENT = os.path.join(ORACLE, "swe_oracle.c")

SOURCES = ["Assigners.cpp", "Bathymetry.cpp", "Fluxes.cpp", "MUSCLObject.cpp", "PointOperations.cpp",
           "Solvers.cpp", "SpaceDisc.cpp", "TimeDisc.cpp", "TriangMesh.cpp", "ValueField.cpp"]

Q1 = ("Bathymetry.cpp",
      "Point Domain::E(NodeTag e) const {\n    return Point{};\n}",
      "Point Domain::E(NodeTag e) const {\n    const auto& ep = m_topology.EdgePoints(e);\n"
      "    return (P(ep[0]) + P(ep[1])) * 0.5;\n}")
Q20 = ("MUSCLObject.cpp",
       "Array<3> hp = wp - b.P(ip);",
       "Array<3> hp = wp - b.P(ip).row(2).transpose();")

CXXFLAGS = ["-std=gnu++17", "-O3", "-DNDEBUG", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-w"]


def reference_root(arg: str | None = None) -> str | None:
    root = arg or os.environ.get("SWE_REFERENCE_ROOT") or "/root/reference"
    return root if os.path.isfile(os.path.join(root, "src", "SpaceDisc.cpp")) else None


def available() -> bool:
    return reference_root() is not None


def _patched(root: str, edit, tag: str) -> str:
    name, old, new = edit
    text = open(os.path.join(root, "src", name)).read()
    if text.count(old) != 1:
        raise RuntimeError(f"{name}: the text to patch was not found exactly once")
    d = os.path.join(OUT, "patched", tag)
    os.makedirs(d, exist_ok=True)
    dst = os.path.join(d, name)
    with open(dst, "w") as fh:
        fh.write(text.replace(old, new))
    return dst


def _compile(args):
    src, obj, lang_flags = args
    cmd = ["g++" if src.endswith(".cpp") else "gcc", *lang_flags, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def _stale(lib: str, root: str) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    deps = [os.path.join(root, "src", s) for s in SOURCES] + [os.path.join(EIGEN, "Eigen", "Dense"), PRELUDE,
                                                               DRIVER, RESTATEMENT, os.path.abspath(__file__)]
    deps += [os.path.join(root, "include", f) for f in os.listdir(os.path.join(root, "include"))]
    return any(os.path.getmtime(d) > t for d in deps)


def build(root: str | None = None, force: bool = False) -> str:
    root = reference_root(root)
    if root is None:
        raise RuntimeError("the reference sources are not present on this machine")
    if not force and not _stale(LIB, root) and not _stale(LIB_Q20LIT, root):
        return LIB
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    inc = ["-I", EIGEN, "-I", os.path.join(root, "include"), "-include", PRELUDE]
    cxx = CXXFLAGS + inc
    q1 = _patched(root, Q1, "q1")
    q20 = _patched(root, Q20, "q20")
    jobs = []
    for s in SOURCES:
        src = {"Bathymetry.cpp": q1, "MUSCLObject.cpp": q20}.get(s, os.path.join(root, "src", s))
        jobs.append((src, os.path.join(OUT, "obj", s + ".o"), cxx))
    jobs.append((os.path.join(root, "src", "MUSCLObject.cpp"), os.path.join(OUT, "obj", "MUSCLObject.q20lit.o"), cxx))
    jobs.append((DRIVER, os.path.join(OUT, "obj", "ref_driver.o"), cxx))
    jobs.append((RESTATEMENT, os.path.join(OUT, "obj", "swe_oracle.o"),
                 ["-std=c11", "-O3", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC"]))
    with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        objs = list(ex.map(_compile, jobs))
    common = [o for o in objs if not o.endswith(("MUSCLObject.cpp.o", "MUSCLObject.q20lit.o"))]
    for lib, muscl in ((LIB, "MUSCLObject.cpp.o"), (LIB_Q20LIT, "MUSCLObject.q20lit.o")):
        tmp = lib + f".tmp{os.getpid()}"
        cmd = ["g++", "-shared", "-fopenmp", "-o", tmp, *common, os.path.join(OUT, "obj", muscl), "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, lib)
    return LIB


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else None, force=True))
