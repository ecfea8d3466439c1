"""GB300-native (sm_103a) implementation of VisACD's visibility-edge
decomposition hot path.

* `visacd_gb300.visacd` (also importable as `visacd`): the reference's pybind
  surface — Mesh, VecArray3d/VecArray3i, MeshList, Config/config, set_seed,
  make_vecarray3i, process.
* `visacd_gb300._native`: ctypes binding of the C ABI (include/visacd_gpu.h).
* `visacd_gb300.meshgen`: seeded synthetic meshes.
"""
