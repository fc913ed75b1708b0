"""Evolution methods: the plug-in point of the mesh path.

Same names and contract as ionization/mesh/evolution_methods.py:16-123:
``evolve(mesh, g, time_step) -> g`` and ``get_evolution_operators``.  On a
device-backed mesh ``evolve`` advances the device-resident wavefunction by one
step with the fused CUDA kernels (the ``g`` argument is the mesh's device
buffer and is returned); ``get_evolution_operators`` returns the host operator
sequence the reference would apply, for inspection and host-side checks.
"""

from .. import units as u
from . import mesh_operators


class EvolutionMethod:
    def evolve(self, mesh, g, time_step):
        """Advance ``mesh`` by one step of ``time_step``; returns the device psi."""
        return mesh._device_evolve(self, time_step)

    def get_evolution_operators(self, mesh, time_step):
        raise NotImplementedError

    def __repr__(self):
        return f"{self.__class__.__name__}()"

    def info(self):
        return self.__class__.__name__


class AlternatingDirectionImplicit(EvolutionMethod):
    """Crank-Nicolson / ADI (evolution_methods.py:46-77): for each H_k of the
    total Hamiltonian, then reversed, alternate (1 - i tau H_k) and
    (1 + i tau H_k)^-1."""

    def get_evolution_operators(self, mesh, time_step):
        tau = time_step / (2 * u.hbar)
        ham_opers = mesh.operators.total_hamiltonian(mesh).operators
        ops = []
        explicit = True
        for oper in list(ham_opers) + list(reversed(ham_opers)):
            if explicit:
                ops.append(
                    mesh_operators.DotOperator(
                        mesh_operators.add_to_diagonal_sparse_matrix_diagonal(-1j * tau * oper.matrix, value=1),
                        wrapping_direction=oper.wrapping_direction,
                    )
                )
            else:
                ops.append(
                    mesh_operators.TDMAOperator(
                        mesh_operators.add_to_diagonal_sparse_matrix_diagonal(1j * tau * oper.matrix, value=1),
                        wrapping_direction=oper.wrapping_direction,
                    )
                )
            explicit = not explicit
        return tuple(ops)


class SplitInteractionOperator(EvolutionMethod):
    """Split operator (evolution_methods.py:80-123): the interaction applied
    as unitary factors around a Crank-Nicolson step of the field-free
    Hamiltonian."""

    def get_evolution_operators(self, mesh, time_step):
        tau = time_step / (2 * u.hbar)
        (cn_oper,) = mesh.operators.internal_hamiltonian(mesh).operators
        return (
            "split_interaction",
            mesh_operators.DotOperator(
                mesh_operators.add_to_diagonal_sparse_matrix_diagonal((-1j * tau) * cn_oper.matrix, value=1),
                wrapping_direction=cn_oper.wrapping_direction,
            ),
            mesh_operators.TDMAOperator(
                mesh_operators.add_to_diagonal_sparse_matrix_diagonal((1j * tau) * cn_oper.matrix, value=1),
                wrapping_direction=cn_oper.wrapping_direction,
            ),
            "split_interaction",
        )


class FourierSplitOperator(EvolutionMethod):
    """Fourier split-step for LineMesh (no counterpart in the reference, whose
    line methods are the Crank-Nicolson ones above):

        P F^-1 K F P,  P = exp(-i tau (V + V_int(t_{n+1}))),  K = exp(-i dt hbar k^2 / 2m)

    with F the discrete Fourier transform over the z mesh, so the line is
    periodic in z (the mask keeps the wavefunction away from the ends).  The
    kinetic factor is exact for band-limited wavefunctions; the splitting error
    is second order in dt.  Requires a power-of-two number of z points."""

    def get_evolution_operators(self, mesh, time_step):
        return ("potential_phase", "fourier_transform", "kinetic_phase", "inverse_fourier_transform",
                "potential_phase")
