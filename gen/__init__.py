"""Seeded synthetic workloads of the projection path (test and benchmark
inputs; not part of the product library).

synth     the five configurations' cases and the parity workloads
geometry  ctypes binding of the C++ cut-cell geometry builder (geometry.cpp)
build     compiles geometry.cpp into gen/_lib/libscf_gen.so
"""
