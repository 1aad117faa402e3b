"""CPU FP64 oracle of quant-iron's state-vector semantics (test infrastructure only).

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py use
this package; the engine never imports, links or calls it.
"""
