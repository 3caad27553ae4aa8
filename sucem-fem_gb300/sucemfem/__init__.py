"""GB300-native drop-in for SUCEM's system-matrix and solve path.

Module paths mirror the reference package (sucemfem.SystemMatrices,
sucemfem.Forms, sucemfem.ProblemConfigurations.*, sucemfem.Sources.*,
sucemfem.Utilities.*).  Meshes are numpy-backed (sucemfem.mesh) and all
assembly and solve work runs in libsucem_gb300.so on the GPU."""
