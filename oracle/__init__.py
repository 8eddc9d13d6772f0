"""CPU oracle for the CKKS engine: TEST INFRASTRUCTURE ONLY.

``pyoracle`` wraps the C restatement of SEAL-4.1-bs arithmetic
(nexus_oracle.c); ``build_ref`` builds the real SEAL library from the NEXUS
sources when they are available.  Only tests, the smoke check and the CPU
baseline of bench.py use this package.
"""
