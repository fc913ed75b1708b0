"""Build product specifications from golden-fixture parameter dicts."""

import numpy as np

import ionization_gb300 as ig
from ionization_gb300 import mesh, potentials, states
from ionization_gb300 import units as u


def pulse(p):
    return potentials.CosSquaredPulse.from_omega_carrier(
        amplitude=p["amplitude"],
        omega_carrier=p["omega_carrier"],
        number_of_cycles=p["number_of_cycles"],
        phase=p["phase"],
        pulse_center=p["pulse_center"],
    )


def product_spec(kind, params, **kw):
    common = dict(
        time_initial=params["time_initial"],
        time_final=params["time_final"],
        time_step=params["time_step"],
        electric_potential=pulse(params["pulse"]),
        store_data_every=params["store_data_every"],
    )
    common.update(kw)
    if kind == "line":
        return mesh.LineSpecification(
            "line",
            z_bound=params["z_bound"],
            z_points=params["z_points"],
            test_mass=params["test_mass"],
            internal_potential=potentials.SoftCoulombPotential(softening_distance=params["softening_distance"]),
            initial_state=states.GaussianState(width=params.get("gaussian_width", 1.0)),
            mask=potentials.AbsoluteRadialCosineMask(**params["mask"]),
            operators=(mesh.LineVelocityGaugeOperators() if params.get("gauge", "length") == "velocity"
                       else mesh.LineLengthGaugeOperators()),
            evolution_method=getattr(mesh, params["method"])(),
            **common,
        )
    if kind == "sh":
        if params.get("gauge", "length") == "velocity":
            common.setdefault("operators", mesh.SphericalHarmonicVelocityGaugeOperators())
        if "kinetic_energy_derivation" in params:
            common.setdefault("operators", mesh.SphericalHarmonicLengthGaugeOperators(
                kinetic_energy_derivation=params["kinetic_energy_derivation"]))
        if "method" in params:
            common.setdefault("evolution_method", getattr(mesh, params["method"])())
        return mesh.SphericalHarmonicSpecification(
            "sh",
            r_points=params["r_points"],
            r_bound=params["r_bound"],
            l_bound=params["l_bound"],
            use_numeric_eigenstates=common.pop("use_numeric_eigenstates", False),
            initial_state=states.HydrogenBoundState(1, 0),
            test_states=[states.HydrogenBoundState(n, l) for n, l in params.get("test_states", [[1, 0]])],
            mask=potentials.RadialCosineMask(**params["mask"]),
            **common,
        )
    if kind == "slice":
        return mesh.SphericalSliceSpecification(
            "slice",
            r_points=params["r_points"],
            r_bound=params["r_bound"],
            theta_points=params["theta_points"],
            initial_state=states.HydrogenBoundState(1, 0),
            test_states=[states.HydrogenBoundState(n, l) for n, l in params["test_states"]],
            mask=potentials.RadialCosineMask(**params["mask"]),
            **common,
        )
    if kind == "rect":
        init = states.TwoDGaussianWavepacket(center_z=params["center_z"], center_x=params["center_x"],
                                             width_z=params["width_z"], width_x=params["width_x"],
                                             k_z=params["k_z"], k_x=params.get("k_x", 0.0))
        return mesh.RectangleSpecification(
            "rect",
            z_points=params["z_points"],
            z_bound=params["z_bound"],
            x_points=params["x_points"],
            x_bound=params["x_bound"],
            internal_potential=potentials.SoftCoulombPotential(softening_distance=params["softening_distance"]),
            initial_state=init,
            test_states=[init],
            mask=potentials.RadialCosineMask(**params["mask"]),
            **common,
        )
    if kind == "cyl":
        return mesh.CylindricalSliceSpecification(
            "cyl",
            z_points=params["z_points"],
            z_bound=params["z_bound"],
            rho_points=params["rho_points"],
            rho_bound=params["rho_bound"],
            initial_state=states.HydrogenBoundState(1, 0),
            test_states=[states.HydrogenBoundState(n, l) for n, l in params["test_states"]],
            **common,
        )
    raise ValueError(kind)


def test_state_order(spec):
    """Product test states are sorted like the reference's (sims.py:530-538)."""
    return [s.tuple for s in spec.test_states]
