"""Writes tests/golden/reference_tests.json: the known-answer values that the reference's own test suite
(kyungminlee/ExactDiagonalization.jl v0.14.3, test/*.jl) asserts for the hot path, transcribed by hand
from those files (each entry names its source file:line).  The reference is Julia and cannot run in
this environment, so these transcribed values are what pins the oracle.

Bit states are written as integers (0b0011 -> 3).  Site and local-state indices are converted to
0-based; everything else is as in the test files.

Run:  python tests/golden/make_golden.py
"""
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))

GOLDEN = {
    "spinhalf_L4_sectors": {
        "source": "test/test_spinhalf.jl:41-47",
        "n_sites": 4,
        # 2Sz -> sorted basis
        "sectors": {"4": [0b0000], "2": [0b0001, 0b0010, 0b0100, 0b1000],
                    "0": [0b0011, 0b0101, 0b0110, 0b1001, 0b1010, 0b1100],
                    "-2": [0b0111, 0b1011, 0b1101, 0b1110], "-4": [0b1111]},
    },
    "spinhalf_L4_full": {
        "source": "test/test_spinhalf.jl:36-38",
        "basis": list(range(16)),
    },
    "spinhalf_L4_sz0": {
        "source": "test/test_hilbert_space_representation.jl:13; test/test_reduced_representation.jl:97",
        "basis": [0b0011, 0b0101, 0b0110, 0b1001, 0b1010, 0b1100],
    },
    "tJ": {
        "source": "test/test_hilbert_space_representation.jl:73-134",
        # sites: [em(0,0), up(1,1), dn(1,-1)], [up, dn], [up, dn]
        "sites": [[[0, 0], [1, 1], [1, -1]], [[1, 1], [1, -1]], [[1, 1], [1, -1]]],
        "sectors": [[2, -2], [2, 0], [2, 2], [3, -3], [3, -1], [3, 1], [3, 3]],
        "all_basis": [0b0000, 0b0001, 0b0010, 0b0100, 0b0101, 0b0110, 0b1000, 0b1001, 0b1010,
                      0b1100, 0b1101, 0b1110],
        "qn_basis": [
            [[2, -2], [0b1100]],
            [[2, 0], [0b0100, 0b1000]],
            [[2, 2], [0b0000]],
            [[3, -3], [0b1110]],
            [[3, -1], [0b0110, 0b1010, 0b1101]],
            [[3, 1], [0b0010, 0b0101, 0b1001]],
            [[3, 3], [0b0001]],
        ],
        "union_qns": [[3, 3], [3, 1]],
        "union_basis": [0b0001, 0b0010, 0b0101, 0b1001],
        "unsorted_input": [0b0101, 0b0001, 0b0010, 0b1001],
    },
    "br_too_small": {
        "source": "test/test_hilbert_space_representation.jl:26-33",
        "n_sites": 9,
        "word_bits": 8,
    },
    "translation_L4": {
        "source": "test/test_symmetry_reduce.jl:33-48",
        # LatticeTools irrep index (1-based) -> representatives; index m+1 is momentum 2 pi m / 4
        "reps_by_irrep_index": {"1": [0b0011, 0b0101], "2": [0b0011], "3": [0b0011, 0b0101], "4": [0b0011]},
    },
    "point_L4": {
        "source": "test/test_symmetry_reduce.jl:104-108 (group {E, -1}: x -> -x, SitePermutation([1,4,3,2]))",
        "inversion_map": [0, 3, 2, 1],
        "irreps": [{"chars": [1, 1], "reps": [0b0011, 0b0101, 0b0110, 0b1010]},
                   {"chars": [1, -1], "reps": [0b0011, 0b0110]}],
    },
    "symmorphic_L4": {
        "source": "test/test_symmetry_reduce.jl:120-132 (translations x inversion)",
        "k0_even_reps": [0b0011, 0b0101],
        "k0_odd_reps": [],
    },
    "convention_L7": {
        "source": "test/test_symmetry_reduce.jl:164-212",
        "n_sites": 7,
        "irrep_index": 2,
        "particle": {"sector": 5, "basis": [1, 2, 4, 8, 16, 32, 64], "reps": [1], "phase_sign": 1},
        "hole": {"sector": -5, "basis": [63, 95, 111, 119, 123, 125, 126], "reps": [63], "phase_sign": -1},
        # psi_k[x] = cis(phase_sign * 2 pi x / 7) / sqrt(7) for x = 0..6 over `basis`
    },
    "reduced_H_L4": {
        "source": "test/test_reduced_representation.jl:13-20, 97, 150-165",
        # j1 = sum_i sum_{j in x,y,z} sigma_j(i) sigma_j(i+1), not simplified; k = 0 (irrep index 1)
        "parent_basis": [0b0011, 0b0101, 0b0110, 0b1001, 0b1010, 0b1100],
        "reps": [0b0011, 0b0101],
        "psis": [[1.0, 0.0, 1.0, 1.0, 0.0, 1.0], [0.0, 1.0, 0.0, 0.0, 1.0, 0.0]],
    },
    "symmetry_apply": {
        "source": "test/test_symmetry_apply.jl:20-31",
        "transop": [1, 2, 3, 0],
        "invop": [0, 3, 2, 1],
        "state_cases": [[0b0001, 0b0010], [0b0101, 0b1010]],
        "pop1": [0b1101, 0b0101, 0b1100, 2.0],
        "pop1_trans": [0b1011, 0b1010, 0b1001, 2.0],
        "pop1_inv": [0b0111, 0b0101, 0b0110, 2.0],
    },
    "bitflip": {
        "source": "test/test_bitflip.jl:33-38",
        "n_sites": 4,
        "perm": [1, 2, 3, 0],
        "cases": {"b0": [0b0001, 0b0001], "b1": [0b0001, 0b1110], "p_b0": [0b0001, 0b0010], "p_b1": [0b0001, 0b1101]},
    },
    "oprep_iterator": {
        "source": "test/test_operator_representation.jl:123-132",
        # op2 = 2 |Up><Dn|_site1 + 3 |Dn><Up|_site1 (0-based site 1) on basis [0b00, 0b01] of a 4-site space
        "basis": [0b00, 0b01],
        "terms": [[0b10, 0b00, 0b10, 2.0], [0b10, 0b10, 0b00, 3.0]],
        "row_targets_invalid": True,
    },
    "out_of_sector": {
        "source": "test/test_operator_representation.jl:275-296",
        # sigma_x on site 1 (0-based) on the L=4 2Sz=0 sector maps every state out of the sector
        "n_sites": 4,
        "site": 1,
        "state_value": [0.0, 2.0],
    },
    "apply_semantics": {
        "source": "test/test_operator_representation.jl:181-272",
        # sigma_+ on site 2 (1-based) of the full L=4 space: kron(s0, s0, s+, s0) in Julia's kron order
        "n_sites": 4,
        "site": 1,
    },
    "frozen_sorted": {
        "source": "test/test_frozensortedarray.jl:5-12",
        "unsorted": [2, 1, 3],
        "duplicates": [1, 1, 2],
    },
}


def main():
    path = os.path.join(HERE, "reference_tests.json")
    with open(path, "w") as f:
        json.dump(GOLDEN, f, indent=1, sort_keys=True)
    print(path)


if __name__ == "__main__":
    main()
