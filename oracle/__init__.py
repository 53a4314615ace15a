"""CPU oracle of the Lambda MIS volumetric path tracer -- test infrastructure only.

Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker; the
product library never links or calls it.
"""
