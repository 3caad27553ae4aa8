"""Convert the reference's own test fixtures into small .npz golden files.

Run where the reference tree is available, with its path as the only
argument; the tests need only the .npz files written here.  Sources:

* sucemfem/ProblemConfigurations/tests/LHS_matrix.npy and RHS_vector.pickle
  (test_EMDrivenProblem.py:64-82): InscribedTet, order 1, f=1e8 Hz, ABC,
  point source at the origin with value [2,-1,3].
* sucemfem/Sources/tests/fillament_source_test_data.pickle
  (test_fillament_source.py:34-69): order-2 filament RHS contributions.
* sucemfem/PostProcessing/tests/data/power_flux_reference_dofs_*.pickle
  (generator power_flux_generate_dofs.py:33-102): order-2 driven solution,
  its DOLFIN XML mesh (coordinates rounded to 6 digits: the mesh the
  reference's power-flux test integrates on; kept as XML text) and the
  test's expected flux (test_power_flux.py:54, SurfaceFlux, and :77,
  VariationalSurfaceFlux).
* sucemfem/PostProcessing/tests/data/reference_surface_ntff-2-*.pickle
  (test_ntff.py:62-92): far fields of the ntff_solution_o2 DOFs evaluated on
  the unshifted centred cube (the test builds get_centred_cube without the
  source translation the generator used).
* reference_variational_ntff-2-*.pickle (test_ntff.py:95-100): the same
  directions by the variational transform.
* functional_tests/data/meshes/rectangular_prism{,_facet_region}.xml: a
  DOLFIN XML mesh and facet mesh function, kept as XML text for the reader
  tests.
* sucemfem/PostProcessing/tests/data/reference_dofs-2-0.149896229-*.pickle
  (generator ntff_generate_dofs.py:40-95): order-2 driven solution of a
  point dipole on a shifted 5^3 cube.
"""
import os
import pickle
import sys

import numpy as np

if len(sys.argv) != 2:
    sys.exit("usage: python make_golden.py <path of the reference checkout>")
REF = sys.argv[1]
OUT = os.path.dirname(os.path.abspath(__file__))


def load_pickle(path):
    with open(path, "rb") as f:
        return pickle.load(f, encoding="latin1")


def main():
    pc = os.path.join(REF, "sucemfem/ProblemConfigurations/tests")
    lhs = np.load(os.path.join(pc, "LHS_matrix.npy"))
    rhs = np.asarray(load_pickle(os.path.join(pc, "RHS_vector.pickle")))
    np.savez_compressed(os.path.join(OUT, "driven_inscribed_tet_o1.npz"),
                        lhs=lhs, rhs=rhs, frequency=1e8,
                        source_coord=np.array([0, 0, 0.]), source_value=np.array([2, -1, 3.]))
    d = load_pickle(os.path.join(REF, "sucemfem/Sources/tests/fillament_source_test_data.pickle"))
    np.savez_compressed(os.path.join(OUT, "fillament_source_o2.npz"),
                        **{k: np.asarray(v) for k, v in d.items()})
    dd = os.path.join(REF, "sucemfem/PostProcessing/tests/data")
    d = load_pickle(os.path.join(dd, "power_flux_reference_dofs_f-1000000000.000000_o-2_s-0.074948_l-0.100000_h-0.166667.pickle"))
    with open(os.path.join(dd, d["meshfile"])) as f:
        mesh_xml = f.read()
    np.savez_compressed(os.path.join(OUT, "power_flux_solution_o2.npz"),
                        x=d["x"], freq=d["freq"], order=d["order"], I=d["I"],
                        source_endpoints=d["source_endpoints"],
                        domain_size=0.25 * 299792458 / 1e9, max_edge_len=299792458 / 1e9 / 6,
                        no_integration_points=100, mesh_xml=np.array(mesh_xml),
                        flux_surface=26.3586862457,
                        flux_variational=26.9015957282 - 7.85747240242e-08j)
    d = load_pickle(os.path.join(dd, "reference_surface_ntff-2-0.149896229-0.0499654096667.pickle"))
    ff = d["ff_result_data"]
    np.savez_compressed(os.path.join(OUT, "surface_ntff_o2.npz"),
                        theta_deg=np.asarray(ff["theta_deg"], dtype=np.float64),
                        phi_deg=np.asarray(ff["phi_deg"], dtype=np.float64),
                        E_ff=np.asarray(ff["E_ff"]),
                        E_theta_analytical=np.asarray(ff["E_theta_analytical"]),
                        rtol=1e-12, atol=1e-7)
    d = load_pickle(os.path.join(dd, "reference_variational_ntff-2-0.149896229-0.0499654096667.pickle"))
    ff = d["ff_result_data"]
    np.savez_compressed(os.path.join(OUT, "variational_ntff_o2.npz"),
                        theta_deg=np.asarray(ff["theta_deg"], dtype=np.float64),
                        phi_deg=np.asarray(ff["phi_deg"], dtype=np.float64),
                        E_ff=np.asarray(ff["E_ff"]), rtol=1e-12, atol=1e-7)
    md = os.path.join(REF, "functional_tests/data/meshes")
    texts = {}
    for key, name in (("mesh_xml", "rectangular_prism.xml"),
                      ("facet_xml", "rectangular_prism_facet_region.xml")):
        with open(os.path.join(md, name)) as f:
            texts[key] = np.array(f.read())
    np.savez_compressed(os.path.join(OUT, "rectangular_prism_xml.npz"), **texts)
    d = load_pickle(os.path.join(dd, "reference_dofs-2-0.149896229-0.0499654096667.pickle"))
    np.savez_compressed(os.path.join(OUT, "ntff_solution_o2.npz"),
                        x=d["x"], freq=d["freq"], order=d["order"],
                        domain_size=d["domain_size"], max_edge_len=d["max_edge_len"],
                        source_value=np.array([0, 0, 1.]) * 299792458 / 1e9 / 1000)


if __name__ == "__main__":
    main()
