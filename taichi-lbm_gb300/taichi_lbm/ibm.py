"""Immersed-boundary coupling (taichi_lbm/ibm.py) is not part of this build:
no example case of the reference uses it.  The names exist so that imports
of the reference's public surface resolve; constructing one raises."""


class _NotBuilt:
    def __init__(self, *args, **kwargs):
        raise NotImplementedError(f"{type(self).__name__} (immersed boundary, taichi_lbm/ibm.py) "
                                  "is not part of this build")


class IBMNodes(_NotBuilt):
    pass


class Sphere(_NotBuilt):
    pass


class SphereIB(_NotBuilt):
    pass


class IBDEMCouplerEngine(_NotBuilt):
    pass


class IBEngine(_NotBuilt):
    pass
