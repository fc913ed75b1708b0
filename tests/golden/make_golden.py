#!/usr/bin/env python
"""Generate golden fixtures by running the REFERENCE ionization library.

This script needs a checkout of the reference, given with ``--ref`` or the
``IONIZATION_REFERENCE`` environment variable; it imports it read-only through ``refstub/loader.py``
(atomic-unit ``simulacra`` stub) and writes ``tests/golden/*.npz``.  The
fixtures are committed; tests only read them.

Cases (reference call sites in parentheses):
  tdma.npz         random complex tridiagonal systems solved by ``cy.tdma``
                   (ionization/cy.pyx:9-50; distribution as tests/conftest.py:4-5)
  line_adi_small   LineMesh + LineLengthGaugeOperators + AlternatingDirectionImplicit
  line_split_small LineMesh + LineLengthGaugeOperators + SplitInteractionOperator
  sh_split_*       SphericalHarmonicMesh + SphericalHarmonicLengthGaugeOperators
                   + SplitInteractionOperator (even L; odd L; odd Nr and odd L)
  cyl_adi_small    CylindricalSliceMesh + CylindricalSliceLengthGaugeOperators + ADI
  line_cfg1_full   the full 1D workload: 4096 points, 4000 steps (optional --full)
  sh_cfg2_full     the full spherical-harmonic workload: Nr=2000, L=41, 20000 steps
                   (optional --full-sh, ~10 min single core)
  cyl_cfg3_full    the full cylindrical workload: 2000 x 1000, 5000 steps
                   (optional --full-cyl, ~1 h single core; psi stored subsampled)
  *_velocity_small  SH (even L; odd Nr and odd L; even Nr and odd L) and line
                   (even and odd z_points) runs in the velocity gauge
                   (SphericalHarmonicVelocityGaugeOperators,
                   LineVelocityGaugeOperators) with SplitInteractionOperator
  sh_adi_small_*   SphericalHarmonicMesh + SphericalHarmonicLengthGaugeOperators
                   + AlternatingDirectionImplicit (even L; odd Nr and odd L)
  rect_adi_small*  RectangleMesh + RectangleLengthGaugeOperators + ADI (96 x 80; 81 x 64)
  slice_adi_small* SphericalSliceMesh + SphericalSliceLengthGaugeOperators + ADI
  sh_numeric_small SH run with use_numeric_eigenstates=True (test states, initial
                   state from eigsh; energies, l and radial vectors recorded)
  *_observables_small  line / SH / cylindrical runs with the ZExpectationValue,
                   RExpectationValue, NormWithinRadius and (SH)
                   NormBySphericalHarmonic datastores
  *_energy_small   line (length and velocity gauge), SH, cylindrical and
                   rectangle runs with the InternalEnergyExpectationValue and
                   TotalEnergyExpectationValue datastores; the SH run also
                   the DirectionalRadialProbabilityCurrent at its final time
  sh_hamiltonian_small  SH split run with kinetic_energy_derivation="hamiltonian"

Each npz holds the spec parameters (``params`` JSON string), the time grid,
the initial and final ``g``, and the Norm / InnerProducts datastore arrays.
"""

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "refstub"))


def _pulse_kwargs(E0, omega, cycles, cep):
    """sin^2-envelope pulse E0 sin^2(pi t/T) cos(w t + cep) as CosSquaredPulse args.

    CosSquaredPulse (potentials/pulses.py:1696-1814) centres the carrier at
    ``pulse_center``; with pulse_center = T/2 the carrier phase must be
    cep + pi * cycles so that E(t) = E0 sin^2(pi t/T) cos(w t + cep).
    """
    T = cycles * 2 * np.pi / omega
    return dict(
        amplitude=E0,
        omega_carrier=omega,
        number_of_cycles=cycles,
        phase=float(np.mod(cep + np.pi * cycles, 2 * np.pi)),
        pulse_center=T / 2,
    )


def build_helpers(ion):
    from ionization import states, potentials

    class GaussianState(states.QuantumState):
        """Normalised-on-mesh Gaussian exp(-(z - z0)^2 / (2 w^2)) (1D)."""

        eigenvalues = states.Eigenvalues.DISCRETE
        binding = states.Binding.BOUND
        derivation = states.Derivation.ANALYTIC

        def __init__(self, width=1.0, center=0.0, amplitude=1):
            self.width = width
            self.center = center
            super().__init__(amplitude=amplitude)

        @property
        def tuple(self):
            return (self.width, self.center)

        def __call__(self, z):
            return np.exp(-((z - self.center) ** 2) / (2 * self.width ** 2)).astype(
                np.complex128
            )

        @property
        def ket(self):
            return "|gauss>"

        @property
        def tex_ket(self):
            return "gauss"

    class AbsRadialCosineMask(potentials.RadialCosineMask):
        """RadialCosineMask evaluated at |r| (absorbs at both ends of a line)."""

        def __call__(self, *, r, **kwargs):
            return super().__call__(r=np.abs(r))

    return GaussianState, AbsRadialCosineMask


def run_and_collect(spec, extra=None, subsample=None):
    sim = spec.to_sim()
    g0 = np.array(sim.mesh.g, copy=True)
    t0 = time.time()
    sim.run()
    elapsed = time.time() - t0
    out = dict(
        times=np.asarray(sim.times),
        data_times=np.asarray(sim.data_times),
        norm=np.asarray(sim.data.norm),
        g_initial=g0,
        g_final=np.asarray(sim.mesh.g),
        elapsed_s=np.float64(elapsed),
    )
    ips = sim.data.inner_products
    keys = list(ips.keys())
    out["inner_products"] = np.array([ips[k] for k in keys])
    out["state_keys"] = np.array([str(k.tuple) for k in keys])
    out["initial_state_overlap"] = np.asarray(sim.data.initial_state_overlap)
    if extra:
        out.update(extra)
    if subsample is not None:
        out["g_initial"] = out["g_initial"][subsample]
        out["g_final"] = out["g_final"][subsample]
    return sim, out


def save(name, params, arrays):
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, params=json.dumps(params), **arrays)
    print(f"wrote {path} ({os.path.getsize(path) / 1024:.1f} KiB)", flush=True)


def gen_tdma(ion):
    from ionization.cy import tdma
    from scipy import sparse

    rng = np.random.default_rng(20261203)
    cases = {}
    sizes = [2, 3, 4, 5, 17, 64, 100, 257, 1000]
    for i, n in enumerate(sizes):
        cs = lambda k: rng.random(k) + 1j * rng.random(k)  # noqa: E731
        a, b, c, d = cs(n - 1), cs(n), cs(n - 1), cs(n)
        dia = sparse.diags([a, b, c], offsets=[-1, 0, 1])
        x = tdma(dia, d)
        # the dia_matrix rows exactly as cy.tdma reads them
        cases[f"n{i}_data"] = np.asarray(dia.data)
        cases[f"n{i}_d"] = d
        cases[f"n{i}_x"] = x
    # a batch of independent lines flattened into one call, the way the mesh
    # operators hand cy.tdma a whole mesh (zero off-diagonals at line ends)
    nl, n = 7, 33
    b = 2.5 + rng.random(nl * n) + 1j * rng.random(nl * n)
    off = rng.random(nl * n - 1) + 1j * rng.random(nl * n - 1)
    off[n - 1 :: n] = 0
    dia = sparse.diags([off, b, off.copy()], offsets=[-1, 0, 1])
    d = rng.random(nl * n) + 1j * rng.random(nl * n)
    cases["batch_data"] = np.asarray(dia.data)
    cases["batch_d"] = d
    cases["batch_x"] = tdma(dia, d)
    cases["batch_shape"] = np.array([nl, n])
    save("tdma", {"sizes": sizes, "seed": 20261203}, cases)


def line_spec(ion, name, z_points, z_bound, steps, dt, pulse, method, mask, store_every, gauge="length"):
    GaussianState, AbsRadialCosineMask = build_helpers(ion)
    import simulacra.units as u

    params = dict(
        z_points=z_points,
        z_bound=z_bound,
        time_initial=0.0,
        time_final=steps * dt,
        time_step=dt,
        softening_distance=float(np.sqrt(2)),
        test_mass=1.0,
        pulse=pulse,
        mask=mask,
        method=method,
        store_data_every=store_every,
        gaussian_width=1.0,
    )
    if gauge != "length":
        params["gauge"] = gauge
    spec = ion.mesh.LineSpecification(
        name,
        z_bound=z_bound,
        z_points=z_points,
        test_mass=u.electron_mass,
        internal_potential=ion.potentials.SoftCoulombPotential(
            softening_distance=np.sqrt(2)
        ),
        initial_state=GaussianState(width=1.0),
        electric_potential=ion.potentials.CosSquaredPulse.from_omega_carrier(**pulse),
        mask=AbsRadialCosineMask(**mask),
        time_initial=0.0,
        time_final=steps * dt,
        time_step=dt,
        operators=ion.mesh.LineVelocityGaugeOperators() if gauge == "velocity" else ion.mesh.LineLengthGaugeOperators(),
        evolution_method=getattr(ion.mesh, method)(),
        store_data_every=store_every,
    )
    return spec, params


def gen_line(ion, full=False):
    pulse = _pulse_kwargs(0.05, 0.057, 4, 0.0)
    mask = dict(inner_radius=80.0, outer_radius=100.0, smoothness=8)
    if not full:
        fast_pulse = _pulse_kwargs(0.1, 0.5, 2, 0.3)
        for method, name in (
            ("AlternatingDirectionImplicit", "line_adi_small"),
            ("SplitInteractionOperator", "line_split_small"),
        ):
            spec, params = line_spec(
                ion, name, 512, 40.0, 600, 0.05, fast_pulse, method,
                dict(inner_radius=30.0, outer_radius=40.0, smoothness=8), 50,
            )
            _, out = run_and_collect(spec)
            save(name, params, out)
    else:
        spec, params = line_spec(
            ion, "line_cfg1_full", 4096, 100.0, 4000, 0.05, pulse,
            "AlternatingDirectionImplicit", mask, 500,
        )
        _, out = run_and_collect(spec)
        save("line_cfg1_full", params, out)


def sh_spec(ion, name, r_points, l_bound, steps, dt, pulse, mask_width, store_every, n_max=3, gauge="length",
            method="SplitInteractionOperator", derivation=None):
    from ionization import states

    r_bound = 0.125 * (r_points - 1)
    r_max = r_bound + 0.125 / 2
    test_states = [states.HydrogenBoundState(n, l) for n in range(1, n_max + 1) for l in range(n)]
    mask = dict(inner_radius=r_max - mask_width, outer_radius=r_max, smoothness=8)
    params = dict(
        r_points=r_points,
        r_bound=r_bound,
        l_bound=l_bound,
        time_initial=0.0,
        time_final=steps * dt,
        time_step=dt,
        pulse=pulse,
        mask=mask,
        store_data_every=store_every,
        test_states=[[s.n, s.l] for s in test_states],
    )
    if gauge != "length":
        params["gauge"] = gauge
    if method != "SplitInteractionOperator":
        params["method"] = method
    if derivation is not None:
        params["kinetic_energy_derivation"] = derivation
    if gauge == "velocity":
        operators = ion.mesh.SphericalHarmonicVelocityGaugeOperators()
    elif derivation is not None:
        operators = ion.mesh.SphericalHarmonicLengthGaugeOperators(
            kinetic_energy_derivation=ion.mesh.KineticEnergyDerivation(derivation))
    else:
        operators = ion.mesh.SphericalHarmonicLengthGaugeOperators()
    spec = ion.mesh.SphericalHarmonicSpecification(
        name,
        r_points=r_points,
        r_bound=r_bound,
        l_bound=l_bound,
        use_numeric_eigenstates=False,
        initial_state=states.HydrogenBoundState(1, 0),
        test_states=test_states,
        electric_potential=ion.potentials.CosSquaredPulse.from_omega_carrier(**pulse),
        mask=ion.potentials.RadialCosineMask(**mask),
        time_initial=0.0,
        time_final=steps * dt,
        time_step=dt,
        operators=operators,
        evolution_method=getattr(ion.mesh, method)(),
        store_data_every=store_every,
    )
    return spec, params


def gen_sh(ion, full=False):
    if not full:
        fast_pulse = _pulse_kwargs(0.1, 0.5, 2, 0.0)
        for name, nr, L in (
            ("sh_split_small_evenL", 160, 8),
            ("sh_split_small_oddL", 160, 11),
            ("sh_split_small_oddNr_oddL", 151, 7),
        ):
            spec, params = sh_spec(ion, name, nr, L, 1250, 0.02, fast_pulse, 5.0, 125)
            _, out = run_and_collect(spec)
            save(name, params, out)
    else:
        pulse = _pulse_kwargs(0.05, 0.057, 6, 0.0)
        spec, params = sh_spec(ion, "sh_cfg2_full", 2000, 41, 20000, 0.02, pulse, 25.0, 1000, n_max=5)
        _, out = run_and_collect(spec)
        save("sh_cfg2_full", params, out)


def gen_velocity(ion):
    """Velocity-gauge split operators: SphericalHarmonicVelocityGaugeOperators
    (mesh_operators.py:1130-1408: l-rotations h1, r/l similarity blocks h2)
    and LineVelocityGaugeOperators (mesh_operators.py:352-427), with
    SplitInteractionOperator; the vector potential is the reference's
    Simpson integral of E over the times so far (pulses.py:58-77)."""
    fast_pulse = _pulse_kwargs(0.1, 0.5, 2, 0.0)
    for name, nr, L in (("sh_velocity_small_evenL", 160, 8), ("sh_velocity_small_oddNr_oddL", 151, 7),
                        ("sh_velocity_small_evenNr_oddL", 160, 11)):
        spec, params = sh_spec(ion, name, nr, L, 500, 0.02, fast_pulse, 5.0, 50, gauge="velocity")
        _, out = run_and_collect(spec)
        save(name, params, out)
    for name, nz in (("line_velocity_small", 512), ("line_velocity_small_odd", 511)):
        spec, params = line_spec(
            ion, name, nz, 40.0, 400, 0.05, _pulse_kwargs(0.1, 0.5, 2, 0.3), "SplitInteractionOperator",
            dict(inner_radius=30.0, outer_radius=40.0, smoothness=8), 50, gauge="velocity",
        )
        _, out = run_and_collect(spec)
        save(name, params, out)


def gen_sh_adi(ion):
    """SphericalHarmonicMesh + SphericalHarmonicLengthGaugeOperators with
    AlternatingDirectionImplicit (evolution_methods.py:46-77 over
    total_hamiltonian, mesh_operators.py:1020-1035): the radial H0 and the
    l-coupling interaction alternate explicit / implicit halves."""
    fast_pulse = _pulse_kwargs(0.1, 0.5, 2, 0.0)
    for name, nr, L in (("sh_adi_small_evenL", 160, 8), ("sh_adi_small_oddNr_oddL", 151, 7)):
        spec, params = sh_spec(ion, name, nr, L, 500, 0.02, fast_pulse, 5.0, 50,
                               method="AlternatingDirectionImplicit")
        _, out = run_and_collect(spec)
        save(name, params, out)


def gen_numeric(ion):
    """SphericalHarmonicSpecification with use_numeric_eigenstates=True
    (meshes.py:1021-1033, 1281-1356): the test states and the initial state
    become numeric eigenstates of each single-l Hamiltonian found by eigsh.
    Records each numeric state's energy, l and radial vector (as the mesh
    uses it), with the run's data."""
    from ionization import states

    fast_pulse = _pulse_kwargs(0.1, 0.5, 2, 0.0)
    nr, L, steps, dt = 300, 6, 300, 0.02
    r_bound = 0.125 * (nr - 1)
    r_max = r_bound + 0.125 / 2
    mask = dict(inner_radius=r_max - 5.0, outer_radius=r_max, smoothness=8)
    params = dict(r_points=nr, r_bound=r_bound, l_bound=L, time_initial=0.0, time_final=steps * dt,
                  time_step=dt, pulse=fast_pulse, mask=mask, store_data_every=50,
                  numeric_eigenstate_max_energy=2.0, numeric_eigenstate_max_angular_momentum=3)
    spec = ion.mesh.SphericalHarmonicSpecification(
        "sh_numeric_small", r_points=nr, r_bound=r_bound, l_bound=L, use_numeric_eigenstates=True,
        numeric_eigenstate_max_energy=2.0, numeric_eigenstate_max_angular_momentum=3,
        initial_state=states.HydrogenBoundState(1, 0),
        electric_potential=ion.potentials.CosSquaredPulse.from_omega_carrier(**fast_pulse),
        mask=ion.potentials.RadialCosineMask(**mask), time_initial=0.0, time_final=steps * dt, time_step=dt,
        operators=ion.mesh.SphericalHarmonicLengthGaugeOperators(),
        evolution_method=ion.mesh.SplitInteractionOperator(), store_data_every=50,
    )
    sim, out = run_and_collect(spec)
    ts = list(sim.spec.test_states)
    out["numeric_energy"] = np.array([s.energy for s in ts])
    out["numeric_l"] = np.array([s.l for s in ts])
    out["numeric_bound"] = np.array([s.binding == states.Binding.BOUND for s in ts])
    out["numeric_g"] = np.array([sim.mesh.get_radial_g_for_state(s) for s in ts])
    save("sh_numeric_small", params, out)


def gen_slice(ion):
    """SphericalSliceMesh + SphericalSliceLengthGaugeOperators + ADI
    (meshes.py:887-983, mesh_operators.py:693-813): the theta kinetic
    operator is a non-symmetric tridiagonal."""
    from ionization import states

    pulse = _pulse_kwargs(0.1, 0.5, 2, 0.3)
    for name, nr, nth in (("slice_adi_small", 96, 64), ("slice_adi_small_odd", 81, 49)):
        test = [states.HydrogenBoundState(1, 0), states.HydrogenBoundState(2, 0), states.HydrogenBoundState(2, 1)]
        params = dict(r_points=nr, r_bound=20.0, theta_points=nth, time_initial=0.0, time_final=10.0,
                      time_step=0.02, pulse=pulse, mask=dict(inner_radius=15.0, outer_radius=20.0, smoothness=8),
                      store_data_every=50, test_states=[[st.n, st.l] for st in test])
        spec = ion.mesh.SphericalSliceSpecification(
            name, r_points=nr, r_bound=20.0, theta_points=nth,
            initial_state=states.HydrogenBoundState(1, 0), test_states=test,
            electric_potential=ion.potentials.CosSquaredPulse.from_omega_carrier(**pulse),
            mask=ion.potentials.RadialCosineMask(inner_radius=15.0, outer_radius=20.0, smoothness=8),
            time_initial=0.0, time_final=10.0, time_step=0.02, store_data_every=50,
        )
        _, out = run_and_collect(spec)
        save(name, params, out)


def rect_spec(ion, name, nz, nx):
    from ionization import states

    pulse = _pulse_kwargs(0.1, 0.5, 2, 0.3)
    params = dict(z_points=nz, z_bound=20.0, x_points=nx, x_bound=16.0, time_initial=0.0, time_final=20.0,
                  time_step=0.05, softening_distance=float(np.sqrt(2)), width_z=1.0, width_x=1.5,
                  center_z=0.5, center_x=-0.25, k_z=0.3, pulse=pulse,
                  mask=dict(inner_radius=12.0, outer_radius=16.0, smoothness=8), store_data_every=50)
    init = states.TwoDGaussianWavepacket(center_z=0.5, center_x=-0.25, width_z=1.0, width_x=1.5, k_z=0.3)
    spec = ion.mesh.RectangleSpecification(
        name, z_points=nz, z_bound=20.0, x_points=nx, x_bound=16.0,
        internal_potential=ion.potentials.SoftCoulombPotential(softening_distance=np.sqrt(2)),
        initial_state=init, test_states=[init],
        electric_potential=ion.potentials.CosSquaredPulse.from_omega_carrier(**pulse),
        mask=ion.potentials.RadialCosineMask(inner_radius=12.0, outer_radius=16.0, smoothness=8),
        time_initial=0.0, time_final=20.0, time_step=0.05, store_data_every=50,
    )
    return spec, params


def gen_rect(ion):
    """RectangleMesh + RectangleLengthGaugeOperators + ADI (meshes.py:430-506,
    mesh_operators.py:430-505): kinetic energies along z (F order) and x
    (C order) in that order, soft-Coulomb V(r) and -z q E(t) split evenly
    between them; a TwoDGaussianWavepacket initial state."""
    for name, nz, nx in (("rect_adi_small", 96, 80), ("rect_adi_small_odd", 81, 64)):
        spec, params = rect_spec(ion, name, nz, nx)
        _, out = run_and_collect(spec)
        save(name, params, out)


def cyl_spec(ion, name, z_points, z_bound, rho_points, rho_bound, steps, dt, pulse, store_every):
    from ionization import states

    test_states = [states.HydrogenBoundState(1, 0), states.HydrogenBoundState(2, 0), states.HydrogenBoundState(2, 1)]
    params = dict(
        z_points=z_points,
        z_bound=z_bound,
        rho_points=rho_points,
        rho_bound=rho_bound,
        time_initial=0.0,
        time_final=steps * dt,
        time_step=dt,
        pulse=pulse,
        store_data_every=store_every,
        test_states=[[s.n, s.l] for s in test_states],
    )
    spec = ion.mesh.CylindricalSliceSpecification(
        name,
        z_points=z_points,
        z_bound=z_bound,
        rho_points=rho_points,
        rho_bound=rho_bound,
        initial_state=states.HydrogenBoundState(1, 0),
        test_states=test_states,
        electric_potential=ion.potentials.CosSquaredPulse.from_omega_carrier(**pulse),
        time_initial=0.0,
        time_final=steps * dt,
        time_step=dt,
        operators=ion.mesh.CylindricalSliceLengthGaugeOperators(),
        evolution_method=ion.mesh.AlternatingDirectionImplicit(),
        store_data_every=store_every,
    )
    return spec, params


def gen_cyl(ion, full=False):
    if not full:
        fast_pulse = _pulse_kwargs(0.1, 0.5, 2, 0.0)
        spec, params = cyl_spec(ion, "cyl_adi_small", 120, 15.0, 60, 15.0, 500, 0.05, fast_pulse, 50)
        _, out = run_and_collect(spec)
        save("cyl_adi_small", params, out)
    else:
        pulse = _pulse_kwargs(0.02, 0.1, 4, 0.0)
        spec, params = cyl_spec(ion, "cyl_cfg3_full", 2000, 100.0, 1000, 100.0, 5000, 0.02, pulse, 500)
        sub = (slice(None, None, 10), slice(None, None, 10))
        params["g_subsample"] = [10, 10]
        _, out = run_and_collect(spec, subsample=sub)
        save("cyl_cfg3_full", params, out)


OBS_RADII = {"line": (-5.0, 0.0, 12.5), "sh": (2.0, 5.0, 12.0), "cyl": (3.0, 7.5)}


def _observable_datastores(ion, kind):
    d = ion.mesh.data if hasattr(ion.mesh, "data") else __import__("ionization.mesh.data").mesh.data
    stores = [d.Fields(), d.Norm(), d.InnerProducts(), d.NormWithinRadius(radii=OBS_RADII[kind])]
    if kind != "line":  # LineLengthGaugeOperators.z/r return tuples: the reference's line <z> raises
        stores += [d.ZExpectationValue(), d.RExpectationValue()]
    # NormBySphericalHarmonic.init reads self.spec before Datastore.init sets
    # it, so the reference cannot run that datastore; its per-l norm is taken
    # from SphericalHarmonicMesh.norm_by_l (meshes.py:1133-1136) after the run
    return stores


def _observable_arrays(sim, kind):
    out = dict(
        radii=np.asarray(OBS_RADII[kind]),
        norm_within_radius=np.array([sim.data.norm_within_radius[r] for r in OBS_RADII[kind]]),
        # the Fields datastore (data.py:152-181): E(t) and A(t) at the data times
        electric_field_amplitude=np.asarray(sim.data.electric_field_amplitude),
        vector_potential_amplitude=np.asarray(sim.data.vector_potential_amplitude),
    )
    if kind != "line":
        out["z_expectation_value"] = np.asarray(sim.data.z_expectation_value)
        out["r_expectation_value"] = np.asarray(sim.data.r_expectation_value)
    if kind == "sh":
        out["norm_by_l_final"] = np.asarray(sim.mesh.norm_by_l())
    return out


def gen_observables(ion):
    """ZExpectationValue, RExpectationValue, NormWithinRadius and (SH)
    NormBySphericalHarmonic datastores (ionization/mesh/data.py:344-464) on
    small line, SH and cylindrical runs."""
    fast_pulse = _pulse_kwargs(0.1, 0.5, 2, 0.0)
    spec, params = line_spec(ion, "line_observables_small", 512, 40.0, 300, 0.05, _pulse_kwargs(0.1, 0.5, 2, 0.3),
                             "SplitInteractionOperator", dict(inner_radius=30.0, outer_radius=40.0, smoothness=8), 25)
    spec.datastores = _observable_datastores(ion, "line")
    spec.datastore_types = tuple(type(ds) for ds in spec.datastores)
    sim, out = run_and_collect(spec)
    out.update(_observable_arrays(sim, "line"))
    save("line_observables_small", params, out)

    spec, params = sh_spec(ion, "sh_observables_small", 160, 11, 500, 0.02, fast_pulse, 5.0, 50)
    spec.datastores = _observable_datastores(ion, "sh")
    spec.datastore_types = tuple(type(ds) for ds in spec.datastores)
    sim, out = run_and_collect(spec)
    out.update(_observable_arrays(sim, "sh"))
    save("sh_observables_small", params, out)

    spec, params = cyl_spec(ion, "cyl_observables_small", 120, 15.0, 60, 15.0, 200, 0.05, fast_pulse, 25)
    spec.datastores = _observable_datastores(ion, "cyl")
    spec.datastore_types = tuple(type(ds) for ds in spec.datastores)
    sim, out = run_and_collect(spec)
    out.update(_observable_arrays(sim, "cyl"))
    save("cyl_observables_small", params, out)


def _energy_datastores(ion):
    m = ion.mesh
    return [m.Fields(), m.Norm(), m.InnerProducts(), m.InternalEnergyExpectationValue(),
            m.TotalEnergyExpectationValue()]


def _run_energy(ion, spec, params, name, extra=None):
    spec.datastores = _energy_datastores(ion)
    spec.datastore_types = tuple(type(ds) for ds in spec.datastores)
    sim, out = run_and_collect(spec)
    out["internal_energy_expectation_value"] = np.asarray(sim.data.internal_energy_expectation_value)
    out["total_energy_expectation_value"] = np.asarray(sim.data.total_energy_expectation_value)
    if extra:
        out.update(extra(sim))
    save(name, params, out)


def _radial_current_final(ion, sim):
    """DirectionalRadialProbabilityCurrent.store (data.py:467-505) at the final
    time.  Two lines of the reference keep that datastore from running as
    written: its init reads self.sim before Datastore.init sets it, and
    get_radial_probability_current_density_mesh__spatial (meshes.py:1358-1371)
    calls r_probability_current__spatial() without its mesh argument.  Here
    the datastore gets sim and spec before init and the operators object a
    bound call that supplies the mesh; the rest is the reference's code."""
    ops = sim.mesh.operators
    meth = type(ops).r_probability_current__spatial
    ops.r_probability_current__spatial = lambda: meth(ops, sim.mesh)
    ds = ion.mesh.DirectionalRadialProbabilityCurrent()
    ds.sim, ds.spec = sim, sim.spec
    ds.init(sim)
    sim.data_time_index = len(sim.data_times) - 1
    ds.store()
    k = sim.data_time_index
    return dict(theta_points=np.int64(sim.spec.theta_points),
                radial_current_pos_z_final=np.asarray(ds.radial_probability_current__pos_z[k]),
                radial_current_neg_z_final=np.asarray(ds.radial_probability_current__neg_z[k]))


def gen_energy(ion):
    """InternalEnergyExpectationValue and TotalEnergyExpectationValue
    (data.py:290-340) on line (length and velocity gauge), SH, cylindrical
    and rectangle runs; the SH run also records the radial probability
    current of DirectionalRadialProbabilityCurrent at its final time."""
    line_mask = dict(inner_radius=30.0, outer_radius=40.0, smoothness=8)
    for gauge, name in (("length", "line_energy_small"), ("velocity", "line_energy_velocity_small")):
        spec, params = line_spec(ion, name, 512, 40.0, 300, 0.05, _pulse_kwargs(0.1, 0.5, 2, 0.3),
                                 "SplitInteractionOperator", line_mask, 25, gauge=gauge)
        _run_energy(ion, spec, params, name)
    fast_pulse = _pulse_kwargs(0.1, 0.5, 2, 0.0)
    spec, params = sh_spec(ion, "sh_energy_small", 160, 11, 500, 0.02, fast_pulse, 5.0, 50)
    _run_energy(ion, spec, params, "sh_energy_small", extra=lambda sim: _radial_current_final(ion, sim))
    spec, params = cyl_spec(ion, "cyl_energy_small", 120, 15.0, 60, 15.0, 200, 0.05, fast_pulse, 25)
    _run_energy(ion, spec, params, "cyl_energy_small")
    spec, params = rect_spec(ion, "rect_energy_small", 96, 80)
    _run_energy(ion, spec, params, "rect_energy_small")


def gen_hamiltonian(ion):
    """SphericalHarmonicLengthGaugeOperators(kinetic_energy_derivation=
    "hamiltonian") with SplitInteractionOperator (mesh_operators.py:863-887):
    the radial kinetic energy of the flattened (l, r) mesh, whose couplings
    also join the last r of each l to the first r of the next.  A short grid
    (64 points, r up to 8) that the pulse drives out to its edge, so that
    those couplings act; the energy datastores ride along."""
    pulse = _pulse_kwargs(0.2, 0.5, 2, 0.0)
    spec, params = sh_spec(ion, "sh_hamiltonian_small", 64, 7, 400, 0.02, pulse, 1.0, 40,
                           derivation="hamiltonian")
    _run_energy(ion, spec, params, "sh_hamiltonian_small")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("IONIZATION_REFERENCE"),
                    help="path of the reference checkout (or set IONIZATION_REFERENCE)")
    ap.add_argument("--only", default=None,
                    help="comma list: tdma,line,sh,cyl,obs,vel,shadi,rect,num,slice,energy,ham")
    ap.add_argument("--full", action="store_true", help="also the full 1D workload")
    ap.add_argument("--full-sh", action="store_true")
    ap.add_argument("--full-cyl", action="store_true")
    args = ap.parse_args()
    if not args.ref:
        ap.error("give the reference checkout with --ref or IONIZATION_REFERENCE")

    from loader import import_reference

    ion = import_reference(args.ref)
    only = set(args.only.split(",")) if args.only else {"tdma", "line", "sh", "cyl", "obs", "vel", "shadi", "rect",
                                                        "num", "slice", "energy", "ham"}
    if "tdma" in only:
        gen_tdma(ion)
    if "line" in only:
        gen_line(ion)
    if "sh" in only:
        gen_sh(ion)
    if "cyl" in only:
        gen_cyl(ion)
    if "obs" in only:
        gen_observables(ion)
    if "vel" in only:
        gen_velocity(ion)
    if "shadi" in only:
        gen_sh_adi(ion)
    if "rect" in only:
        gen_rect(ion)
    if "num" in only:
        gen_numeric(ion)
    if "slice" in only:
        gen_slice(ion)
    if "energy" in only:
        gen_energy(ion)
    if "ham" in only:
        gen_hamiltonian(ion)
    if args.full:
        gen_line(ion, full=True)
    if args.full_sh:
        gen_sh(ion, full=True)
    if args.full_cyl:
        gen_cyl(ion, full=True)


if __name__ == "__main__":
    main()
