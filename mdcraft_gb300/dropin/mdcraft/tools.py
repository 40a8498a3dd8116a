"""mdcraft.tools (python/mdcraft/tools/_tools.cxx): the thread pool handle.
The GPU engine needs no host threads; the object keeps the API and the
count semantics of tools::Threads (mdcraft/tools/threads.cxx:10-12,58-74):
the count is capped at the host's hardware threads, off() leaves one and
on() restores the cap."""
import os


class Threads:
    def __init__(self, count: int = 100000, comm=None):
        self._max = max(1, os.cpu_count() or 1)
        self._count = max(1, min(int(count), self._max))

    @property
    def count(self) -> int:
        return self._count

    def on(self, count: int = 0):
        self._count = self._max

    def off(self):
        self._count = 1
