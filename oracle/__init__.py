"""CPU checkers for the GB300 library.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline / reference legs of bench.py.  The product library never loads
anything from this package.

* ``oracle.restatement`` -- ctypes wrapper of liboracle.so, the C restatement
  of grav_sim's hot path (grav_oracle.c);
* ``oracle.reference``   -- ctypes wrapper of grav_sim itself compiled from
  its own sources into oracle/_ref/ (only where those sources exist).
"""
