"""CPU oracle for the state-vector engine: TEST INFRASTRUCTURE ONLY.

A C (OpenMP) restatement of the reference's Numba kernels plus a ctypes front end.
Only the tests, the smoke check and the CPU legs of the benchmark use it, as the
checker and the CPU baseline; the engine itself never imports it.
"""
