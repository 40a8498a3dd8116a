"""mdcraft.solver.thermostat (python/mdcraft/solver/thermostat/_thermostat.cxx).
Constructible so that scripts which make one but do not pass it to a solver
run; passing one to a solver raises (the GPU path is NVE)."""


class Langevin:
    def __init__(self, beta=0.0, temperature=0.0, time_step=0.0, heat_x=1, heat_y=1, heat_z=1,
                 Ux=0.0, Uy=0.0, Uz=0.0, *rest):
        self.beta, self.temperature, self.time_step = beta, temperature, time_step
        self.heat = (heat_x, heat_y, heat_z)
        self.U = (Ux, Uy, Uz)
