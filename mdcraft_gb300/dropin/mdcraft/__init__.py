"""GPU drop-in for MDcraft's Python package (python/mdcraft): the modules and
class names a driver script imports — mdcraft.tools.Threads,
mdcraft.data.Atoms, mdcraft.lattice.Domain, mdcraft.neibs.VerletList,
mdcraft.solver.{Single, Multi}, mdcraft.solver.potential.{EAM, LJsCut},
mdcraft.solver.boundary.Periodic, mdcraft.solver.stepper.Verlet — backed by
libmdg on the GPU. Put this directory (mdcraft_gb300/dropin) on sys.path
instead of the reference's build.

Atoms keep the reference's host-side record array (`Atoms.data`, the 208-byte
Atom with nested r/v/f/V fields); every call that reads or writes atoms
copies them to the device, runs there and copies them back, so scripts that
read or modify `atoms.data` between calls see the reference's semantics.
"""
