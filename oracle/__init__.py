"""CPU oracle of the GB300 stencil engine — TEST INFRASTRUCTURE ONLY.

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg, as the checker.  The product (formura_gb300) never imports it.
"""
