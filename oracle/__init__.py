"""Parity oracle package -- TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline and
reference legs as the checker; never imported by the product package.
"""
