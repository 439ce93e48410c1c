#!/usr/bin/env python3
"""Build the reference's own lduMatrix solver code as a CPU oracle library.

This is test infrastructure, not product code.  It compiles, from the
OpenFOAM-dev sources where they lie (read-only), the three libraries the
lduMatrix solver path needs:

* ``src/OpenFOAM``        (lduMatrix, solvers, smoothers, GAMG, polyMesh, ...)
* ``src/OSspecific/POSIX`` (signals, clocks, file ops)
* ``src/Pstream/dummy``   (serial reduce = no-op)

into one shared object ``oracle/_ref/libOpenFOAM.so``, without wmake: the
source lists are read from each ``Make/files``, a flat include farm of
symlinks (what wmake calls ``lnInclude``) is made under ``oracle/_ref``, and a
generated Makefile compiles every translation unit with the flags of
``wmake/rules/linux64Gcc/c++`` + ``c++Opt`` (``-std=c++14 -O3 -DWM_DP
-DWM_LABEL_SIZE=32 -DNoRepository``).  ``global/global.Cver`` is compiled as
plain C++ (its VERSION_STRING/BUILD_STRING placeholders stay literal).

The harness ``oracle/ref_harness.C`` (our own code) is then linked against it.
Outputs go only to ``oracle/_ref/``; nothing is written to the reference tree.

Usage: python oracle/build_ref.py [--ref DIR] [-j N]   (DIR defaults to $OPENFOAM_REF_DIR)
"""
import argparse
import os
import re
import subprocess
import sys

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from refpath import REF_ROOT  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")

LIBS = [
    ("OpenFOAM", "src/OpenFOAM"),
    ("POSIX", "src/OSspecific/POSIX"),
    ("Pstream", "src/Pstream/dummy"),
]

HDR_EXT = (".H", ".C", ".h", ".c", ".hxx", ".cxx", ".hpp", ".cpp", ".type")

CXXFLAGS = [
    "-std=c++14", "-m64", "-O3", "-fPIC",
    "-Dlinux64", "-DWM_ARCH_OPTION=64", "-DWM_DP", "-DWM_LABEL_SIZE=32",
    "-DNoRepository", "-ftemplate-depth-256",
    "-Wno-deprecated-declarations", "-w",
]


def parse_make_files(path):
    """Return the list of source files named by a wmake Make/files."""
    vars_ = {"WM_PRECISION_OPTION": "DP", "WM_ARCH": "linux64"}
    srcs = []
    stack = []
    with open(path) as fh:
        for raw in fh:
            line = raw.split("#", 1)[0].strip()
            if not line:
                continue
            for _ in range(4):
                line = re.sub(r"\$\((\w+)\)",
                              lambda mm: vars_.get(mm.group(1), ""), line)
            m = re.match(r'^(ifeq|ifneq)\s+"([^"]*)"\s+"([^"]*)"', line)
            if m:
                eq = m.group(2) == m.group(3)
                stack.append(eq if m.group(1) == "ifeq" else not eq)
                continue
            if line.startswith("else"):
                stack[-1] = not stack[-1]
                continue
            if line.startswith("endif"):
                stack.pop()
                continue
            if not all(stack):
                continue
            m = re.match(r"^([A-Za-z_][A-Za-z0-9_]*)\s*=\s*(.*)$", line)
            if m:
                if m.group(1) != "LIB":
                    vars_[m.group(1)] = m.group(2).strip()
                continue
            srcs.append(line)
    return srcs


def make_farm(src_dir, farm):
    os.makedirs(farm, exist_ok=True)
    seen = {}
    for root, _dirs, files in os.walk(src_dir):
        if "/Make" in root or root.endswith("Make"):
            continue
        for f in sorted(files):
            if f.endswith(HDR_EXT):
                if f in seen:
                    continue
                seen[f] = os.path.join(root, f)
    for f, p in seen.items():
        dst = os.path.join(farm, f)
        if os.path.islink(dst) or os.path.exists(dst):
            if os.path.realpath(dst) == p:
                continue
            os.remove(dst)
        os.symlink(p, dst)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=REF_ROOT)
    ap.add_argument("-j", type=int, default=os.cpu_count() or 4)
    args = ap.parse_args()
    ref = os.path.abspath(args.ref)
    if not os.path.isdir(os.path.join(ref, "src/OpenFOAM")):
        print("reference sources not found at", ref)
        return 1
    os.makedirs(OUT, exist_ok=True)
    farms = {}
    for name, rel in LIBS:
        farms[name] = os.path.join(OUT, "lnInclude", name)
        make_farm(os.path.join(ref, rel), farms[name])
    inc = ["-I" + farms["OpenFOAM"], "-I" + farms["POSIX"]]

    objs = []
    rules = []
    for name, rel in LIBS:
        sdir = os.path.join(ref, rel)
        for s in parse_make_files(os.path.join(sdir, "Make/files")):
            src = os.path.join(sdir, s)
            obj = os.path.join(OUT, "obj", name, s.rsplit(".", 1)[0] + ".o")
            lang = "-x c++ " if s.endswith(".Cver") else ""
            objs.append(obj)
            rules.append(
                f"{obj}: {src}\n\t@mkdir -p $(dir $@)\n"
                f"\t@$(CXX) $(FLAGS) -I{sdir} {lang}-c $< -o $@\n"
            )
    lib = os.path.join(OUT, "libOpenFOAM.so")
    harness_src = os.path.join(HERE, "ref_harness.C")
    harness = os.path.join(OUT, "ref_harness")
    # the OpenFOAM-side plugin of the solver library, built against this
    # reference build so that a test can load it as controlDict's libs
    # entry would (the harness's plugin mode)
    repo = os.path.dirname(HERE)
    plugin_src = os.path.join(repo, "openfoam-dev_gb300", "plugin", "cudaLduSolvers.C")
    solver_lib_dir = os.path.join(repo, "openfoam-dev_gb300", "lib")
    plugin = os.path.join(OUT, "libcudaLduSolvers_OpenFOAM.so")
    mk = os.path.join(OUT, "Makefile")
    with open(mk, "w") as fh:
        fh.write("CXX = g++\n")
        fh.write("FLAGS = " + " ".join(CXXFLAGS + inc) + "\n")
        fh.write(f"all: {harness} {plugin}\n")
        fh.write(f"{lib}: {' '.join(objs)}\n"
                 f"\t$(CXX) -shared -fuse-ld=bfd -o $@ $^ -lz -lpthread -ldl -lm\n")
        fh.write(f"{harness}: {harness_src} {os.path.join(HERE, 'harness_io.H')} {lib}\n"
                 f"\t$(CXX) $(FLAGS) -o $@ {harness_src} -L{OUT} -lOpenFOAM "
                 f"-Wl,-rpath,{OUT} -lz -lpthread -ldl -lm\n")
        fh.write(f"{plugin}: {plugin_src} {os.path.join(repo, 'include', 'cfx.h')} {lib}\n"
                 f"\t$(CXX) $(FLAGS) -shared -I{os.path.join(repo, 'include')} -o $@ {plugin_src} "
                 f"-L{OUT} -lOpenFOAM -L{solver_lib_dir} -lcudaLduSolvers "
                 f"-Wl,-rpath,{OUT} -Wl,-rpath,{solver_lib_dir}\n")
        fh.write("\n".join(rules))
    r = subprocess.call(["make", "-f", mk, f"-j{args.j}", "-k"])
    return r


if __name__ == "__main__":
    sys.exit(main())
