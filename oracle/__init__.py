"""Test oracle for the GB300 sort library (TEST INFRASTRUCTURE ONLY).

Only tests/, the smoke check and bench.py's CPU-baseline leg use this package.
"""
