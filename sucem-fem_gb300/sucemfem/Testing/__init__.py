"""Testing helpers of the reference's sucemfem.Testing package."""
