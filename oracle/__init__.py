"""Oracle: CPU restatement of the reference's assemble-and-solve path.

Test infrastructure only.  Imported by tests/, by __graft_entry__.smoke() and by
the CPU-baseline leg of bench.py, always as the checker; the product library
(muscade.jl_gb300/) never imports, links or calls anything here.
"""
