"""Stand-in for roma: fixtures pass explicit 4x4 matrices, so rotation
conversions are never called; any call raises."""


def _unavailable(*a, **k):
    raise RuntimeError("roma is not available; pass explicit matrices")


euler_to_rotmat = rotmat_to_euler = unitquat_to_rotmat = quat_wxyz_to_xyzw = _unavailable
special_procrustes = rotvec_to_rotmat = rotmat_to_rotvec = rotmat_geodesic_distance = _unavailable
