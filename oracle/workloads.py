"""ORACLE — test infrastructure only.

Seeds and length models of the benchmark workloads, for code that generates
them through the oracle library (oracle/synth_oracle.c) without loading the
product package.  They equal siml_gb300.synthetic's constants
(tests/test_compiler.py checks both the constants and the bytes)."""

UNIFORM_20_90 = 0
LOGNORMAL_45 = 1
BIMODAL_35_110 = 2
CHEM_45 = 3

SEED_ALLPAIRS = 20260001
SEED_DB_1M = 20260002
SEED_RAGGED = 20260004
SEED_SERVING = 20260005
SEED_CHEM = 20260006
