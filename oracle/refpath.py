"""Where the reference's sources are read from (test infrastructure only).

The OpenFOAM-dev tree is taken from the environment variable
OPENFOAM_REF_DIR; without it, from the mount the oracle build recipes use.
Nothing on a GPU run reads it: the GPU tests and the bench use the prebuilt
oracle and the committed fixtures.
"""
import os

REF_ROOT = os.environ.get("OPENFOAM_REF_DIR") or "/root/reference"


def sources_present(root=None):
    """True when the reference's OpenFOAM sources are readable at root."""
    return os.path.isdir(os.path.join(root or REF_ROOT, "src", "OpenFOAM"))
