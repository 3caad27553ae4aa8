"""Analytical reference solutions (sucemfem/Testing/Analytical)."""
