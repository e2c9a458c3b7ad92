"""Test oracle for ubootgl_gb300 -- TEST INFRASTRUCTURE ONLY.

The CPU restatement (ubg_oracle.c) and the reference build (ref/, outputs in
_ref/) exist to check the CUDA path.  Only tests/, __graft_entry__.smoke()
and the CPU-baseline / reference legs of bench.py may import this package;
the product package ubootgl_gb300 never does.
"""
