"""Measured errors of the full-size parity tests, collected during a pytest session and
printed by conftest.py's terminal summary (one "PARITY {...}" line per result)."""
RECORDS = []
