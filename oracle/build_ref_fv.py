#!/usr/bin/env python3
"""Build the reference's finite-volume library for the assembly oracle.

Test infrastructure, not product code.  After ``build_ref.py`` (libOpenFOAM),
this compiles, from the OpenFOAM-dev sources where they lie (read-only), the
libraries ``fvm::ddt`` / ``fvm::div`` / ``fvm::laplacian`` need:

* ``src/fileFormats``, ``src/surfMesh``, ``src/triSurface``,
  ``src/meshTools``, ``src/finiteVolume``

into ``oracle/_ref/libfiniteVolume.so`` with the same flags and include farms
as ``build_ref.py``, then links ``oracle/fv_harness.C`` (our own code) against
both libraries.  The flex-generated ASCII STL readers (``*.L``) are not
compiled; the link leaves their two symbols unresolved in the shared library
(nothing on the assembly path reads STL).  Outputs go only to
``oracle/_ref/``.

Usage: python oracle/build_ref_fv.py [--ref DIR] [-j N] [--lib-only]   (DIR defaults to $OPENFOAM_REF_DIR)
"""
import argparse
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import build_ref as br  # noqa: E402

OUT = br.OUT
FV_LIBS = [
    ("fileFormats", "src/fileFormats"),
    ("surfMesh", "src/surfMesh"),
    ("triSurface", "src/triSurface"),
    ("meshTools", "src/meshTools"),
    ("finiteVolume", "src/finiteVolume"),
]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=br.REF_ROOT)
    ap.add_argument("-j", type=int, default=os.cpu_count() or 4)
    ap.add_argument("--lib-only", action="store_true", help="build the library, not the harness")
    args = ap.parse_args()
    ref = os.path.abspath(args.ref)
    if not os.path.exists(os.path.join(OUT, "libOpenFOAM.so")):
        print("build libOpenFOAM first: python oracle/build_ref.py")
        return 1
    farms = {}
    for name, rel in br.LIBS + FV_LIBS:
        farms[name] = os.path.join(OUT, "lnInclude", name)
        br.make_farm(os.path.join(ref, rel), farms[name])
    inc = ["-I" + farms[n] for n, _ in br.LIBS + FV_LIBS if n != "Pstream"]
    objs, rules = [], []
    for name, rel in FV_LIBS:
        sdir = os.path.join(ref, rel)
        for s in br.parse_make_files(os.path.join(sdir, "Make/files")):
            if not s.endswith(".C"):
                continue  # flex (.L) sources: not on the assembly path
            src = os.path.join(sdir, s)
            obj = os.path.join(OUT, "objfv", name, s.rsplit(".", 1)[0] + ".o")
            objs.append(obj)
            rules.append(f"{obj}: {src}\n\t@mkdir -p $(dir $@)\n\t@$(CXX) $(FLAGS) -I{sdir} -c $< -o $@\n")
    lib = os.path.join(OUT, "libfiniteVolume.so")
    harness_src = os.path.join(HERE, "fv_harness.C")
    harness = os.path.join(OUT, "fv_harness")
    mk = os.path.join(OUT, "Makefile.fv")
    with open(mk, "w") as fh:
        fh.write("CXX = g++\n")
        fh.write("FLAGS = " + " ".join(br.CXXFLAGS + inc) + "\n")
        fh.write(f"all: {harness}\n")
        fh.write(f"{lib}: {' '.join(objs)}\n"
                 f"\t$(CXX) -shared -o $@ $^ -L{OUT} -lOpenFOAM -Wl,-rpath,{OUT}\n")
        fh.write(f"{harness}: {harness_src} {os.path.join(HERE, 'harness_io.H')} {lib}\n"
                 f"\t$(CXX) $(FLAGS) -o $@ {harness_src} -L{OUT} -lfiniteVolume -lOpenFOAM "
                 f"-Wl,-rpath,{OUT} -Wl,--unresolved-symbols=ignore-in-shared-libs -lz -lpthread -ldl -lm\n")
        fh.write("".join(rules))
    r = subprocess.run(["make", "-f", mk, f"-j{args.j}", lib if args.lib_only else "all"], cwd=OUT)
    return r.returncode


if __name__ == "__main__":
    sys.exit(main())
