"""CPU oracle of the OLDG field step: test infrastructure only.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs use
this package, and only as the checker or the timed CPU baseline; the product
(libtwoldg and the twoldg package) never imports it.
"""
