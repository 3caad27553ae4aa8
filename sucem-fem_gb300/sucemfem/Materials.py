"""Material regions -> per-cell coefficient arrays.

Same interface and errors as sucemfem/Materials.py:30-150; the DG0
functions of the reference become plain float64 arrays of one value per
cell (``MaterialFunctionFactory`` builds them with one vectorised lookup
instead of a Python loop over cells)."""
import numpy as np

from . import Consts

mu0 = Consts.mu0
eps0 = Consts.eps0


class MaterialProperties:
    allowed_properties_defaults = {"eps_r": 1.0, "mu_r": 1.0}

    def __init__(self):
        for prop, val in self.allowed_properties_defaults.items():
            setattr(self, prop, val)

    def init_values(self, **kwargs):
        for prop, val in kwargs.items():
            if prop not in self.allowed_properties_defaults:
                raise ValueError("Unknown material property")
            setattr(self, prop, val)

    def set_eps_r(self, eps_r):
        self.eps_r = eps_r

    def set_mu_r(self, mu_r):
        self.mu_r = mu_r

    def get_eps_r(self):
        return self.eps_r

    def get_mu_r(self):
        return self.mu_r

    def get_mu_r_inv(self):
        return 1 / self.get_mu_r()

    def get_eps(self):
        return eps0 * self.eps_r

    def get_mu(self):
        return mu0 * self.mu_r


class MaterialPropertiesFactory:
    def __init__(self, material_regions):
        self.material_properties = {}
        if material_regions is None:
            self.material_properties[0] = MaterialProperties()
        else:
            for region_no, property_values in material_regions.items():
                mp = MaterialProperties()
                mp.init_values(**property_values)
                self.material_properties[region_no] = mp

    def get_material_properties(self):
        return self.material_properties


class MaterialFunctionFactory:
    def __init__(self, region_material_properties, region_meshfunction, mesh):
        self.region_material_properties = region_material_properties
        self.mesh = mesh
        if region_meshfunction is None:
            regions = np.zeros(mesh.num_cells(), dtype=np.int64)
        elif hasattr(region_meshfunction, "array"):
            regions = np.asarray(region_meshfunction.array(), dtype=np.int64)
        else:
            regions = np.asarray(region_meshfunction, dtype=np.int64)
        self.regions = regions

    def get_material_functions(self, *property_names):
        out = {}
        keys = np.array(sorted(self.region_material_properties), dtype=np.int64)
        uniq, inv = np.unique(self.regions, return_inverse=True)
        for u in uniq:
            if int(u) not in self.region_material_properties:
                raise ValueError("Material number %d not found" % int(u))
        for pname in property_names:
            getter = "get_" + pname
            vals = np.array([float(getattr(self.region_material_properties[int(u)], getter)())
                             for u in uniq], dtype=np.float64)
            out[pname] = vals[inv.reshape(-1)]
        return out
