"""Parity helpers for the tests (the definitions live in foort_gb300.accuracy)."""
from foort_gb300.accuracy import (BOUNDARY_DELTA, DISCRETE, MIN_DISCRETE_AGREEMENT,  # noqa: F401
                                  discrete_mismatch, endpoint_rel_err, explain_mismatches, outcome, summarize)
