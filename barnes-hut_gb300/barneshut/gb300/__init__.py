"""Native layer of the GB300 implementation: the ctypes binding of
libbh_gb300.so, particle-file I/O and the seeded workload generators."""
