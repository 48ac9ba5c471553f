"""CPU oracle of the RayTracer per-pixel loop (test infrastructure, never used by the renderer).

oracle.port wraps oracle/src/rt_oracle.cpp, a restatement of the reference's algorithm that is
checked against the reference itself (oracle/ref builds it from its sources; the fixtures it
produced live in tests/golden).
"""
