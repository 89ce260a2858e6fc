"""CPU oracle of the rasteriser and pose path — TEST INFRASTRUCTURE ONLY.

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, and
there only as the checker. Nothing in the product package imports it.
"""
