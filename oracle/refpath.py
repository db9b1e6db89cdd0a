"""Where the reference nii2mesh tree is — TEST INFRASTRUCTURE ONLY.

Used by the recipes that compile the reference (oracle/build_ref.sh, called by
``__graft_entry__.build``), by the scripts that generate the golden fixtures
and by the CPU tests that compare the oracle with the reference directly.
Nothing in the product reads the reference.

``N2M_REFERENCE`` names the reference project's root directory (the one
holding ``src/`` and ``data/``).  Without it, a checkout named ``reference``
beside this repository is used when one exists; otherwise there is no
reference tree and everything that needs it is skipped.
"""
import os
from pathlib import Path

REPO = Path(__file__).resolve().parents[1]


def reference_root():
    """The reference project's root directory, or None when there is none."""
    env = os.environ.get("N2M_REFERENCE")
    cand = Path(env) if env else REPO.parent / "reference"
    return cand if (cand / "src" / "meshify.c").exists() else None


def reference_src():
    """The reference's src/ directory, or None."""
    r = reference_root()
    return r / "src" if r else None


def reference_data():
    """The reference's data/ directory, or None."""
    r = reference_root()
    return r / "data" if r else None
