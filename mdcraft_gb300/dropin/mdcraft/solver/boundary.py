"""mdcraft.solver.boundary.Periodic (python/mdcraft/solver/boundary/_boundary.cxx)."""


class Periodic:
    def __init__(self, domain):
        self.domain = domain
