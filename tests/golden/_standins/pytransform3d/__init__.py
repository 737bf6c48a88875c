"""Minimal stand-in for pytransform3d: only what the distance3d reference
imports at module level on the GJK / EPA / AABB-tree path. Used only by the
golden-vector generator in this folder."""
