"""The reference's MEX gateway run on the host (test infrastructure: see build.py)."""
