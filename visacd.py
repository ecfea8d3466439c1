"""`import visacd` — the reference's Python module name, served by this
project's GB300 implementation (the pybind11 module visacd_gb300.visacd).

Same surface as the reference (lib/bindings.cpp:14-70): Mesh, VecArray3d,
VecArray3i, MeshList, Config, make_vecarray3i, set_seed, config, ProcessResult,
process.
"""
from visacd_gb300.visacd import *  # noqa: F401,F403
from visacd_gb300.visacd import config  # noqa: F401  (the process-wide Config, by reference)
