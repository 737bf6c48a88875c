"""Empty stand-in: distance3d.broad_phase imports this module at load time."""


class Sphere:  # pragma: no cover - never instantiated
    pass


class Box:  # pragma: no cover
    pass


class Cylinder:  # pragma: no cover
    pass


class Mesh:  # pragma: no cover
    pass
