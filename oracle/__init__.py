"""CPU oracle -- test infrastructure only.

A C++ restatement of ZisaFVM's per-step path (``zfvm_oracle.cpp``) used by the
tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``.
The product package never imports this module.
"""
