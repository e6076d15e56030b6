"""Where the reference's sources are, for the test-infrastructure builds that
compile them (the reference harness, the Energybase adapter check).

Looked up in this order:
  1. $FG_REFERENCE_DIR (a Faunus checkout with include/faunus and src/);
  2. baseline/_ref/faunus, a copy of the few source folders those builds need,
     made by ``make -C oracle/ref stage REF=<checkout>`` (git-ignored: it is an
     install of the reference next to the repository, not part of it);
  3. none: every build and test that needs the reference is skipped.
Nothing in the product reads this.
"""
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STAGED = os.path.join(ROOT, "baseline", "_ref", "faunus")


def _valid(d):
    return bool(d) and os.path.isdir(os.path.join(d, "include", "faunus")) and os.path.isdir(os.path.join(d, "src"))


def reference_dir():
    """The reference checkout to compile against, or None."""
    env = os.environ.get("FG_REFERENCE_DIR")
    if _valid(env):
        return os.path.abspath(env)
    if _valid(STAGED):
        return STAGED
    return None
