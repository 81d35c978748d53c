"""Where the reference checkout is, for the recipes that read it (the
fixture generators under tests/golden/, the reference build, tests that
read the reference's own data files).

REF_ROOT names the checkout (REF_SRC its src/ directory for the build
recipe). Unset, the recipes look in the one place the development
container mounts it; None means absent, and callers skip.
"""
import os

_CONTAINER_CHECKOUT = "/root/reference"


def ref_root():
    """The reference checkout, or None when it is not on this machine."""
    root = os.environ.get("REF_ROOT")
    if root is None and "REF_SRC" in os.environ:
        root = os.path.dirname(os.path.normpath(os.environ["REF_SRC"]))
    if root is None:
        root = _CONTAINER_CHECKOUT
    return root if os.path.isdir(root) else None


def ref_src():
    """The reference's src/ directory, or None."""
    if "REF_SRC" in os.environ:
        return os.environ["REF_SRC"] if os.path.isdir(os.environ["REF_SRC"]) else None
    root = ref_root()
    return os.path.join(root, "src") if root else None


def ref_file(*parts):
    """A file of the reference checkout, or None when absent."""
    root = ref_root()
    if root is None:
        return None
    p = os.path.join(root, *parts)
    return p if os.path.exists(p) else None
