"""Import the unmodified reference package (dtmm) for golden-vector generation.

Test infrastructure only.  The reference is pure Python + numba; numba and
matplotlib are absent here, so ``_shim/`` supplies pure-Python stand-ins.
numpy 2 removed ``np.alltrue`` (used by the reference's ``mode.fft_mask``), so
it is aliased to ``np.all``.  Byte-code writing is disabled so that nothing is
written into the (read-only) reference tree, and HOME points at a scratch
directory because the reference copies its ini file into ``~/.dtmm``.
"""
import os
import sys
import tempfile

import numpy as np

_SHIM = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_shim")


def reference_root():
    """The reference checkout named by ``DTMM_REFERENCE_ROOT`` (required: a
    checkout elsewhere must not silently import nothing, or another dtmm)."""
    root = os.environ.get("DTMM_REFERENCE_ROOT")
    if not root:
        raise ImportError("set DTMM_REFERENCE_ROOT to the reference checkout (the directory holding dtmm/) "
                          "to generate golden fixtures")
    if not os.path.isdir(os.path.join(root, "dtmm")):
        raise ImportError("DTMM_REFERENCE_ROOT=%s holds no dtmm/ package" % root)
    return root


def load_reference():
    """Return the imported reference ``dtmm`` module (double precision)."""
    if "dtmm" in sys.modules:
        return sys.modules["dtmm"]
    root = reference_root()
    sys.dont_write_bytecode = True
    os.environ.setdefault("DTMM_DOUBLE_PRECISION", "1")
    home = tempfile.mkdtemp(prefix="dtmm_home_")
    os.makedirs(os.path.join(home, ".dtmm"), exist_ok=True)
    os.environ["HOME"] = home
    if not hasattr(np, "alltrue"):
        np.alltrue = np.all
    for p in (_SHIM, root):
        if p not in sys.path:
            sys.path.insert(0, p)
    import dtmm  # noqa: E402

    dtmm.conf.set_verbose(0)
    return dtmm
