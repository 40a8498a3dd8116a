"""mdcraft.tools (python/mdcraft/tools/_tools.cxx): the thread pool handle.
The GPU engine needs no host threads; the object only keeps the API."""


class Threads:
    def __init__(self, count: int = 1, comm=None):
        self.count = count

    def on(self, count: int = 0):
        pass

    def off(self):
        pass
