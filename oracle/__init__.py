"""ORACLE — CPU restatement of the reference's generated programs (elastic and acoustic).

Test infrastructure only: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline / reference arms of bench.py, where it checks or times; it is
never the thing measured on the GPU.  The product (opesci-fd_gb300/) never
imports it.

  cpp_emitter.py      emits the reference-shaped C++/OpenMP program of an
                      elastic (StaggeredGrid) model
  regular_emitter.py  the same for an acoustic (RegularGrid) model
  run.py              compiles (g++, reference flags) and runs them
  Makefile            builds the reference's own benchmarks/test3d.cpp and its
                      opesciHandy.cpp/opesciIO.cpp (resampling, SEG-Y reader,
                      with handy_shim.cpp) into _ref/ for fixture generation
"""
