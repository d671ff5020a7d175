"""Locating and importing the reference torchtree (pure Python, CPU).

TEST/BENCH INFRASTRUCTURE ONLY: used by ``tests/`` and by ``bench.py``'s CPU
legs, never by the package.

Two places are searched, in order:

* ``TORCHTREE_REFERENCE``: a torchtree source tree (the directory holding
  ``torchtree/`` and, for the known-answer tests, ``data/``);
* ``baseline/_ref`` beside this repository: an unmodified copy of torchtree
  1.0.2 installed there with ``pip install --no-deps --target baseline/_ref``
  (git-ignored; it carries the package only, no ``data/``).

torchtree imports dendropy at module load; ``oracle/_stub`` provides the three
names it needs.
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

REPO = Path(__file__).resolve().parents[1]
STUB = REPO / "oracle" / "_stub"
INSTALLED = REPO / "baseline" / "_ref"


def source_root() -> Path | None:
    """The torchtree source tree named by TORCHTREE_REFERENCE, if it exists."""
    env = os.environ.get("TORCHTREE_REFERENCE")
    if env and (Path(env) / "torchtree").is_dir():
        return Path(env)
    return None


def data_dir() -> Path | None:
    """The reference's ``data/`` folder (only a source tree has one)."""
    root = source_root()
    if root is not None and (root / "data").is_dir():
        return root / "data"
    return None


def torchtree_root() -> Path | None:
    root = source_root()
    if root is not None:
        return root
    if (INSTALLED / "torchtree").is_dir():
        return INSTALLED
    return None


def import_torchtree():
    """Import torchtree from its source tree or the installed copy; the module, or None."""
    root = torchtree_root()
    if root is None:
        return None
    for path in (str(STUB), str(root)):
        if path not in sys.path:
            sys.path.insert(0, path)
    try:
        import torchtree
    except ImportError:
        return None
    return torchtree


def describe() -> str:
    root = torchtree_root()
    if root is None:
        return "absent"
    return "source tree (TORCHTREE_REFERENCE)" if root == source_root() else "installed copy (baseline/_ref)"
