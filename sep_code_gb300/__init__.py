"""sep_code_gb300: GB300-native (sm_103a) 3D acoustic Born / RTM propagation.

The product is the native library ``_build/libsepx.so`` (C ABI in
``include/sepx.h``, a drop-in for SEP_Code's ``Born/gpu_funcs_3d.h``); this
package holds its sources (``csrc/``), the build recipe and a thin Python face.
"""
from pathlib import Path

PACKAGE_DIR = Path(__file__).resolve().parent
LIB_PATH = PACKAGE_DIR / "_build" / "libsepx.so"

__all__ = ["PACKAGE_DIR", "LIB_PATH"]
