"""The reference's end-to-end DMRG cases with their golden energies.

Every case is restated from
``tests/test_algorithm/test_two_site_update_finite_vmps.cc`` of gqmps2:
model, initial product state, SweepParams and the energy asserted there.
"""
from mps2_gb300 import hamiltonians as H


def cases():
    N = 6
    pairs2d = [(0, 1), (0, 2), (1, 3), (2, 3), (2, 4), (3, 5), (4, 5)]
    return {
        # name: (builder, labels, (sweeps, Dmin, Dmax, trunc, lanc_err, lanc_max), golden, tol, line)
        "1DIsing": (lambda: H.heisenberg_pairs(N, [(i, i + 1, 1.0) for i in range(N - 1)], ising_only=True),
                    [i % 2 for i in range(N)], (4, 1, 10, 1e-5, 1e-7, 200), -0.25 * (N - 1), 1e-10, 151),
        "1DHeisenberg": (lambda: H.heisenberg_chain(N), [i % 2 for i in range(N)],
                         (4, 8, 8, 1e-9, 1e-7, 200), -2.493577133888, 1e-12, 212),
        "2DHeisenberg": (lambda: H.heisenberg_pairs(N, [(a, b, 1.0) for a, b in pairs2d]),
                         [i % 2 for i in range(N)], (4, 8, 8, 1e-9, 1e-7, 200), -3.129385241572, 1e-12, 280),
        "TjSystem2U1Symm.1DCase": (lambda: H.tj_bonds(4, [(i, i + 1) for i in range(3)]), [2, 1, 2, 0],
                                   (11, 8, 8, 1e-9, 1e-8, 20), -6.947478526233, 1e-10, 576),
        "TjSystem2U1Symm.2DCase": (lambda: H.tj_bonds(4, [(0, 1), (0, 2), (2, 3), (1, 3)]), [2, 0, 1, 2],
                                   (10, 8, 8, 1e-9, 1e-8, 20), -8.868563739680, 1e-10, 636),
        "HubbardSystem.2Dcase": (H.hubbard_2x2_reference, [1 if i % 2 == 0 else 2 for i in range(4)],
                                 (10, 16, 16, 1e-9, 1e-8, 20), -2.828427124746, 1e-10, 950),
        "KondoInsulatorSystem.doublechain": (H.kondo_double_chain, [i % 2 for i in range(8)],
                                             (5, 64, 64, 1e-9, 1e-8, 20), -3.180025784229132, 1e-10, 1112),
    }
