"""Correctness oracle for the cpic time step (test infrastructure only)."""
