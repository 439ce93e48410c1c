"""GB300-native lduMatrix linear solvers (cudaPCG, cudaPBiCGStab, cudaGAMG).

The solver library is ``lib/libcudaLduSolvers.so`` (CUDA kernels for sm_103a
plus the host C++ solvers, exported through the C ABI in
``include/cfx.h``).  This Python package only loads it:

* ``build``  compiles the shared objects in-tree (nvcc / g++);
* ``ldu``    binds the C ABI with ctypes and mirrors OpenFOAM's
             ``lduMatrix::solver::New(...)->solve(psi, source)`` interface;
* ``cases``  builds seeded synthetic LDU systems (hex boxes, Laplacian,
             upwind convection-diffusion, Cuthill-McKee renumbering).

The directory name is not a Python identifier; import it through
``load_package()`` in ``__graft_entry__`` (registered as ``openfoam_dev_gb300``).
"""
import os

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(PKG_DIR, "lib")
CSRC_DIR = os.path.join(PKG_DIR, "csrc")
REPO_DIR = os.path.dirname(PKG_DIR)
INCLUDE_DIR = os.path.join(REPO_DIR, "include")
