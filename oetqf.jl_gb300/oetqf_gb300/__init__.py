"""oetqf_gb300: the GB300 (sm_103a) earthquake-cycle hot path of Oetqf.jl behind a C ABI.

Host-side mirror of the reference API: meshes (src/BEM/mesh.jl), properties
(src/BEM/property.jl), stress_greens_function (src/BEM/GF.jl), assemble and the ODE right-hand
side (src/BEM/equation.jl), and an on-device adaptive integrator. Compute runs in libgbcycle.so.
"""
from .mesh import (BEMHex8Mesh, RectOkadaMesh, gauss1_quadrature, gauss_product_quadrature, gen_hex8_box,
                   gen_mesh, get_quadrature, gmsh_quadrature, sincosd)
from .persist import load_greens_functions, save_greens_functions
from .property import (CompositePowerLawViscosityProperty, DilatancyProperty, PowerLawViscosityProperty,
                       RateStateQuasiDynamicProperty, dϵ_dt, dϵ_dt_composite, load_property, save_property)

import unicodedata as _ud

__all__ = ["BEMHex8Mesh", "RectOkadaMesh", "gen_mesh", "gen_hex8_box", "gauss1_quadrature", "gauss_product_quadrature",
           "sincosd", "RateStateQuasiDynamicProperty", "PowerLawViscosityProperty", "CompositePowerLawViscosityProperty",
           "DilatancyProperty", "dϵ_dt", "dϵ_dt_composite", "stress_greens_function",
           "StrikeSlip", "DipSlip", "assemble", "solve", "ArrayPartition", "GB300Model", "ODEProblem",
           "save_property", "load_property", "save_greens_functions", "load_greens_functions", "gmsh_quadrature",
           "get_quadrature", "wsolve", "Sweep"]
# identifiers are NFKC-normalised (ϵ -> ε); keep the exported names in that form
__all__ = [_ud.normalize("NFKC", n) for n in __all__]


def __getattr__(name):
    # GPU-facing pieces load libgbcycle.so lazily so mesh/property code works without a GPU
    if name in ("stress_greens_function", "StrikeSlip", "DipSlip"):
        from . import greens
        return getattr(greens, name)
    if name in ("assemble", "solve", "ArrayPartition", "GB300Model", "ODEProblem"):
        from . import equation
        return getattr(equation, name)
    if name == "wsolve":
        from . import io
        return io.wsolve
    if name == "Sweep":
        from . import sweep
        return sweep.Sweep
    raise AttributeError(name)
