"""GB300-native (sm_103a) implementation of MeshODE's per-iteration
deformation hot path: distance-field build, DistanceFieldLoss and
RigidEdgeLoss forward/backward, and the Adam update, behind the reference's
``pyDeform`` API (``meshode_gb300.pyDeform``) and its autograd layers
(``meshode_gb300.layers``).  All compute runs in libmeshode.so
(meshode_gb300/csrc, C ABI in include/meshode.h).
"""
__version__ = "0.1.0"
