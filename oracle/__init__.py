"""
The oracle for the FDTD time-stepping path — TEST INFRASTRUCTURE, never part of the product.

  fdtd_port.c / fdtd_port_body.h / port.py   C restatement of the reference kernels
                                              (float32 bit-exact with them; float64 = the
                                              FP64 oracle; plus diagonal mu and Bloch coupling)
  ref_harness.py                              the reference's own Simulation and rendered
                                              kernel text run on the CPU (needs its source tree)
  ref_replay.py                               those rendered kernels replayed where the tree
                                              is absent (oracle/_ref/, generated)

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import this package.
"""
