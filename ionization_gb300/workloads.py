"""Named synthetic workloads (seeded), used by the benchmark and tests.

* ``line_softcore_4096``: 1D line, 4096 points on [-100, 100], soft-core
  V = -1/sqrt(z^2 + 2), Gaussian start, sin^2 pulse E0 0.05 / w 0.057 /
  4 cycles, dt 0.05 x 4000 steps, cos^(1/8) mask on the outer 20 a0 of each
  side, Crank-Nicolson (ADI), complex128.
* ``sh_hydrogen_2000x41``: spherical harmonic, Nr 2000 at dr 0.125, l < 41,
  hydrogen 1s, pulse 0.05 / 0.057 / 6 cycles, dt 0.02 x 20000 steps, radial
  mask on the outer 25 a0, split operator, complex128.
* ``cyl_hydrogen_2000x1000``: cylindrical slice 2000 (z in [-100, 100]) x
  1000 (rho in (0, 100]), hydrogen 1s, pulse 0.02 / 0.1 / 4 cycles,
  dt 0.02 x 5000 steps, ADI, complex128.
* ``uneven_sh_sweep``: 512 spherical-harmonic simulations drawn from
  SeedSequence(20261203).spawn(512): r_max ~ U[100, 400] (Nr = round(r_max /
  0.125)), l_max ~ U{20..80}, E0 log-uniform [0.005, 0.1], w ~ U[0.03, 0.2],
  2..10 cycles, CEP ~ U[0, 2 pi); hydrogen 1s, dt 0.02 x 10000 steps, mask on
  the outer 25 a0, complex64 state.
* ``line_softcore``: soft-core lines of any length at the 4096-point line's
  spacing.
* ``poisson_scan_parameters``: the served scan mix (ionization_gb300.serve):
  Poisson arrivals, lines of 2048-16384 points and SH meshes of Nr 1000-4000,
  l_max 20-100, 2000-50000 steps, 80 % complex64 arithmetic (residual form).
"""

import numpy as np

DR = 0.125


def __getattr__(name):  # torch-dependent modules load lazily
    if name in ("mesh", "potentials", "states"):
        import importlib

        return importlib.import_module(f"ionization_gb300.{name}")
    raise AttributeError(name)


def _mods():
    from . import mesh, potentials, states

    return mesh, potentials, states


def sin2_pulse(E0, omega, cycles, cep=0.0):
    mesh, potentials, states = _mods()
    return potentials.CosSquaredPulse.from_sin2_envelope(E0, omega, cycles, cep)


def hydrogen_test_states(n_max=5):
    mesh, potentials, states = _mods()
    return [states.HydrogenBoundState(n, l) for n in range(1, n_max + 1) for l in range(n)]


def line_softcore_4096(steps=4000, precision="c128", store_data_every=-1, **kw):
    mesh, potentials, states = _mods()
    return mesh.LineSpecification(
        "line_softcore_4096",
        z_bound=100.0,
        z_points=4096,
        test_mass=1.0,
        internal_potential=potentials.SoftCoulombPotential(softening_distance=np.sqrt(2)),
        initial_state=states.GaussianState(width=1.0),
        electric_potential=sin2_pulse(0.05, 0.057, 4),
        mask=potentials.AbsoluteRadialCosineMask(inner_radius=80.0, outer_radius=100.0, smoothness=8),
        time_initial=0.0,
        time_final=steps * 0.05,
        time_step=0.05,
        evolution_method=mesh.AlternatingDirectionImplicit(),
        store_data_every=store_data_every,
        precision=precision,
        **kw,
    )


def sh_spec(name, r_points, l_bound, E0, omega, cycles, cep, steps, dt=0.02, precision="c128",
            store_data_every=-1, n_max=5, mask_width=25.0, **kw):
    mesh, potentials, states = _mods()
    r_bound = DR * (r_points - 1)
    r_max = r_bound + DR / 2
    return mesh.SphericalHarmonicSpecification(
        name,
        r_points=r_points,
        r_bound=r_bound,
        l_bound=l_bound,
        use_numeric_eigenstates=False,
        initial_state=states.HydrogenBoundState(1, 0),
        test_states=hydrogen_test_states(min(n_max, l_bound)),
        electric_potential=sin2_pulse(E0, omega, cycles, cep),
        mask=potentials.RadialCosineMask(inner_radius=r_max - mask_width, outer_radius=r_max, smoothness=8),
        time_initial=0.0,
        time_final=steps * dt,
        time_step=dt,
        store_data_every=store_data_every,
        precision=precision,
        **kw,
    )


def sh_hydrogen_2000x41(steps=20000, precision="c128", **kw):
    return sh_spec("sh_hydrogen_2000x41", 2000, 41, 0.05, 0.057, 6, 0.0, steps, precision=precision, **kw)


def cyl_hydrogen_2000x1000(steps=5000, store_data_every=-1, **kw):
    mesh, potentials, states = _mods()
    T = 4 * 2 * np.pi / 0.1
    return mesh.CylindricalSliceSpecification(
        "cyl_hydrogen_2000x1000",
        z_points=2000,
        z_bound=100.0,
        rho_points=1000,
        rho_bound=100.0,
        initial_state=states.HydrogenBoundState(1, 0),
        test_states=[states.HydrogenBoundState(1, 0), states.HydrogenBoundState(2, 0), states.HydrogenBoundState(2, 1)],
        electric_potential=potentials.CosSquaredPulse.from_omega_carrier(
            amplitude=0.02, omega_carrier=0.1, number_of_cycles=4, phase=float(np.mod(4 * np.pi, 2 * np.pi)),
            pulse_center=T / 2),
        time_initial=0.0,
        time_final=steps * 0.02,
        time_step=0.02,
        store_data_every=store_data_every,
        **kw,
    )


def uneven_sh_parameters(n_sims=512, seed=20261203):
    """Per-simulation parameters of the uneven sweep, one child seed each."""
    out = []
    for i, child in enumerate(np.random.SeedSequence(seed).spawn(n_sims)):
        rng = np.random.default_rng(child)
        r_max = rng.uniform(100.0, 400.0)
        l_max = int(rng.integers(20, 81))
        E0 = float(np.exp(rng.uniform(np.log(0.005), np.log(0.1))))
        omega = float(rng.uniform(0.03, 0.2))
        cycles = int(rng.integers(2, 11))
        cep = float(rng.uniform(0.0, 2 * np.pi))
        out.append(dict(index=i, r_points=int(round(r_max / DR)), l_bound=l_max + 1, E0=E0, omega=omega,
                        cycles=cycles, cep=cep))
    return out


def uneven_sh_sweep(n_sims=512, seed=20261203, steps=10000, precision="c64", store_data_every=-1, n_max=5,
                    subset=None, **kw):
    params = uneven_sh_parameters(n_sims, seed)
    if subset is not None:
        params = [params[i] for i in subset]
    return [
        sh_spec(f"uneven_sh_{p['index']:03d}", p["r_points"], p["l_bound"], p["E0"], p["omega"], p["cycles"],
                p["cep"], steps, precision=precision, store_data_every=store_data_every, n_max=n_max, **kw)
        for p in params
    ]


LINE_DZ = 200.0 / 4095  # the grid spacing of the 4096-point line on [-100, 100]


def line_softcore(name, z_points, E0, omega, cycles, cep, steps, dt=0.05, precision="c128", store_data_every=-1,
                  evolution_method=None, **kw):
    """Soft-core line of ``z_points`` at the spacing of the 4096-point line
    (z_bound grows with the point count), Gaussian start, sin^2 pulse, cos^(1/8)
    mask on the outer 20 % of each side, Crank-Nicolson (ADI) by default."""
    mesh, potentials, states = _mods()
    z_bound = LINE_DZ * (z_points - 1) / 2
    return mesh.LineSpecification(
        name,
        z_bound=z_bound,
        z_points=z_points,
        test_mass=1.0,
        internal_potential=potentials.SoftCoulombPotential(softening_distance=np.sqrt(2)),
        initial_state=states.GaussianState(width=1.0),
        electric_potential=sin2_pulse(E0, omega, cycles, cep),
        mask=potentials.AbsoluteRadialCosineMask(inner_radius=0.8 * z_bound, outer_radius=z_bound, smoothness=8),
        time_initial=0.0,
        time_final=steps * dt,
        time_step=dt,
        evolution_method=evolution_method or mesh.AlternatingDirectionImplicit(),
        store_data_every=store_data_every,
        precision=precision,
        **kw,
    )


def poisson_scan_parameters(n_requests=100, rate=20.0, seed=20261204, line_fraction=0.5, c64_fraction=0.8,
                            c64_precision="c64x"):
    """The served scan mix: Poisson arrivals at ``rate`` per second; each
    request a soft-core line (2048-16384 points) or a hydrogen
    spherical-harmonic mesh (Nr 1000-4000, l_max 20-100), with a pulse drawn
    as in the uneven sweep, 2000-50000 steps, complex64 arithmetic with
    probability ``c64_fraction`` else complex128.  The complex64 requests use
    ``c64_precision``: "c64x" (the residual-compensated state that holds the
    1e-6 population bound) or "c64"."""
    rng = np.random.default_rng(seed)
    out, t = [], 0.0
    for i in range(n_requests):
        t += float(rng.exponential(1.0 / rate))
        kind = "line" if rng.random() < line_fraction else "sh"
        precision = c64_precision if rng.random() < c64_fraction else "c128"
        steps = int(rng.integers(2000, 50001))
        E0 = float(np.exp(rng.uniform(np.log(0.005), np.log(0.1))))
        omega = float(rng.uniform(0.03, 0.2))
        cycles = int(rng.integers(2, 11))
        cep = float(rng.uniform(0.0, 2 * np.pi))
        if kind == "line":
            points, l_bound = int(rng.integers(2048, 16385)), 0
        else:
            points, l_bound = int(rng.integers(1000, 4001)), int(rng.integers(20, 101)) + 1
        out.append(dict(id=i, arrival=t, kind=kind, precision=precision, steps=steps, points=points,
                        l_bound=l_bound, E0=E0, omega=omega, cycles=cycles, cep=cep))
    return out
