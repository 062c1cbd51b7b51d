"""Parity oracle for the voxelhashmt depth-fusion path (test infrastructure only)."""
