"""Write tests/golden/reference_kat.json.

The reference (Merzbild.jl, Julia) cannot run in this environment (no Julia
toolchain, no network).  Its deterministic known-answer tests are therefore
transcribed here: each scenario rebuilds the inputs exactly as the reference
test constructs them and records the values the reference test asserts.  The
file:line of every source assertion is stored next to it.

Scenarios whose inputs the reference draws from an RNG use only RNG-independent
fields (positions are overwritten by the test before the checked operation).

Run:  python tests/golden/make_golden.py
"""
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))

AR_MASS = 66.3e-27   # data/particles.toml ["Ar"] mass
HE_MASS = 6.65e-27   # data/particles.toml ["He"] mass


def particle(w, v, x):
    return [float(w)] + [float(a) for a in v] + [float(a) for a in x]


def octant_particle(octant, v_val, w=1.0, x=(1.0, -10.0, 3.0), v0=(0.0, 0.0, 0.0)):
    # create_particle_in_octant, test/test_octree_merging.jl:3-23
    vz = v_val if octant >= 5 else -v_val
    vx = -v_val if octant % 2 == 1 else v_val
    vy = v_val if octant in (3, 4, 7, 8) else -v_val
    return particle(w, (vx + v0[0], vy + v0[1], vz + v0[2]), x)


def scen_grid_sorting():
    # test/test_grid_sorting.jl:8-67: Grid1DUniform(8, 2), 8 particles whose
    # positions are overwritten to x = 0.99 * 8 * (9 - i) / 8; y carries the
    # particle's physical id so a device run can recover the permutation.
    Fnum = 1e10 / 4
    parts = [particle(Fnum, (0, 0, 0), (0.99 * 8.0 * (9.0 - i) / 8, float(i), 0.0)) for i in range(1, 9)]
    return {
        "name": "grid_sorting_coarse_fine_uneven",
        "source": "test/test_grid_sorting.jl:8-235",
        "Fnum": Fnum,
        "particles": parts,
        "steps": [
            {"op": "sort_grid", "L": 8.0, "nx": 2,
             "pia_before": {"all_in_cell": [1, 2], "cells": [[1, 4], [5, 8]]},
             "expect_index": [5, 6, 7, 8, 1, 2, 3, 4],
             "expect_indexer": [[4, 1, 4, 4, 0, -1, 0], [4, 5, 8, 4, 0, -1, 0]],
             "source": "test/test_grid_sorting.jl:37-54"},
            {"op": "sort_grid", "L": 8.0, "nx": 4,
             "pia_before": {"note": "all 8 in cell 1 group1", "cells": [[1, 8], None, None, None]},
             "expect_index": [7, 8, 5, 6, 3, 4, 1, 2],
             "expect_indexer": [[2, 1 + 2 * c, 2 + 2 * c, 2, 0, -1, 0] for c in range(4)],
             "source": "test/test_grid_sorting.jl:98-125"},
            {"op": "reset_index_and_x", "x": [6.75] * 4 + [2.5] + [0.5] * 3,
             "then": "sort_grid", "L": 8.0, "nx": 4,
             "expect_index": [6, 7, 8, 5, 1, 2, 3, 4],
             "expect_counts": [3, 1, 0, 4], "expect_starts": [1, 4, 0, 5], "expect_ends": [3, 4, -1, 8],
             "expect_n": [3 * Fnum, 1 * Fnum, 0.0, 4 * Fnum], "n_tol": "2eps",
             "source": "test/test_grid_sorting.jl:145-187"},
            {"op": "reset_index_and_cells", "cell": [4, 4, 4, 4, 2, 1, 1, 1],
             "then": "sort_cells",
             "expect_index": [6, 7, 8, 5, 1, 2, 3, 4],
             "expect_counts": [3, 1, 0, 4], "expect_starts": [1, 4, 0, 5], "expect_ends": [3, 4, -1, 8],
             "source": "test/test_grid_sorting.jl:189-235"},
        ],
    }


def scen_convection():
    # test/test_convection_1D.jl:9-73 and :271-321
    parts = [
        particle(1.0, (-1.25, -1.5, 4.0), (23.0, -8.0, 7.5)),
        particle(2.0, (11.0, -3.0, 1.0), (49.0, 6.0, -3.0)),
        particle(3.0, (-20.0, 0.0, 2.0), (17.0, 1.0, 3.0)),
        particle(4.0, (-49.0, -20.0, 13.0), (1.55, -1.0, 9.0)),
    ]
    return {
        "name": "convection_specular_4particles",
        "source": "test/test_convection_1D.jl:9-73,271-321",
        "mass": AR_MASS,
        "L": 50.0, "nx": 100, "dt": 2.0,
        "walls": [1.0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0],
        "particles": parts,
        "pia": {"cell": 1, "n": 4},
        "expect_cells_after_convect": [42, 59, 47, 8],
        "expect_index_after_sort": [4, 1, 3, 2],
        "expect_sorted": [
            {"x": [3.55, -1.0, 9.0], "x_tol": 3.65e-15, "v": [-49.0, -20.0, 13.0], "w": 4.0},
            {"x": [20.5, -8.0, 7.5], "x_tol": "2eps", "v": [-1.25, -1.5, 4.0], "w": 1.0},
            {"x": [23.0, 1.0, 3.0], "x_tol": "2eps", "v": [20.0, 0.0, 2.0], "w": 3.0},
            {"x": [29.0, 6.0, -3.0], "x_tol": "2eps", "v": [-11.0, -3.0, 1.0], "w": 2.0},
        ],
        "expect_n_by_cell": {"8": 4.0, "42": 1.0, "47": 3.0, "59": 2.0},
        "source_asserts": "test/test_convection_1D.jl:39-73,301-321",
    }


def scen_convection_noncontiguous():
    # test/test_convection_1D.jl:213-269: 30 particles, indexer points at
    # group1 [1,10] and group2 [26,30] of cell 2; only those 15 move.
    parts = []
    for i in range(1, 31):
        if 11 <= i <= 25:
            parts.append(particle(10000.0, (-1000.0, 0.0, 0.0), (0.75, 0.0, 0.0)))
        else:
            parts.append(particle(1.0, (1.0, 0.0, 0.0), (0.75, 0.0, 0.0)))
    return {
        "name": "convection_noncontiguous",
        "source": "test/test_convection_1D.jl:213-269",
        "mass": AR_MASS,
        "L": 50.0, "nx": 100, "dt": 1.0,
        "walls": [1.0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0],
        "particles": parts,
        "indexer_cell2": [15, 1, 10, 10, 26, 30, 5],
        "n_total": 15,
        "expect_before": {"n_cell2": 15.0, "v1_cell2": 1.0},
        "expect_after": {"n_cell4": 15.0, "v1_cell4": 1.0, "others_zero": True},
    }


def scen_collision_utils():
    # test/test_collision_utils.jl:8-40
    return {
        "name": "collision_utils_com_g",
        "source": "test/test_collision_utils.jl:8-40",
        "p1": particle(1e10, (2.0, 1.0, 0.0), (0, 0, 0)),
        "p2": particle(1e10, (0.0, -1.0, -1.0), (0, 0, 0)),
        "expect_mu": [0.5, 0.5],
        "expect_v_com": [1.0, 0.0, -0.5],
        "expect_g": 3.0,
        "g_after_scatter_tol": "2.1eps",
    }


def scen_octree_merge():
    # test/test_octree_merging.jl:25-44 (create_24_3particles_in_octant) and
    # the assertions at :78-163, :165-203, :205-272, :274-290.
    def make24(weights):
        ps = []
        for octant in range(1, 9):
            for dv in (-0.5, 0.5, 0.0):
                ps.append(octant_particle(octant, 9.0 - octant + dv, w=octant * weights[octant - 1]))
        return ps

    ones = [1.0] * 8
    mean_expect = []
    for i in range(1, 9):
        vzs = 1 if i >= 5 else -1
        vxs = -1 if i % 2 == 1 else 1
        vys = 1 if i in (3, 4, 7, 8) else -1
        mean_expect.append([(9.0 - i) * vxs, (9.0 - i) * vys, (9.0 - i) * vzs])
    return {
        "name": "octree_merge_24",
        "source": "test/test_octree_merging.jl:25-290",
        "mass": AR_MASS,
        "particles24": make24(ones),
        "split_once": {"init_bin_bounds": "C", "expect_Nbins": 8, "expect_np": [3] * 8,
                       "expect_w": [3.0 * i for i in range(1, 9)], "expect_v_mean": mean_expect,
                       "expect_x_mean": [1.0, -10.0, 3.0], "tol": 1e-14,
                       "source": "test/test_octree_merging.jl:74-119"},
        "merge16": {"target": 16, "expect_Nbins": 8, "expect_n_total": 16, "expect_depth": 1,
                    "cons_tol": {"n": "eps", "T": 1e-14, "v": 1e-14},
                    "source": "test/test_octree_merging.jl:129-145"},
        "merge2_after16": {"target": 2, "expect_Nbins": 1, "expect_n_total": 2, "expect_w_each": 0.5 * 108.0,
                           "source": "test/test_octree_merging.jl:147-163"},
        "zero_weight_last": {"weights": [1, 1, 1, 1, 1, 1, 1, 0], "target": 16, "expect_n_total": 14,
                             "particles": make24([1, 1, 1, 1, 1, 1, 1, 0]),
                             "source": "test/test_octree_merging.jl:165-203"},
        "zero_weight_two_groups": {"weights": [1, 1, 0, 1, 0, 1, 1, 0], "target": 16, "expect_n_total": 10,
                                   "particles": make24([1, 1, 0, 1, 0, 1, 1, 0]),
                                   "indexer": [24, 1, 7, 7, 8, 24, 17],
                                   "source": "test/test_octree_merging.jl:205-272"},
        "two_particles": {"particles": [octant_particle(1, 9.0 - 1 - 0.5, w=1), octant_particle(1, 9.0 - 1 + 0.5, w=2)],
                          "target": 16, "expect_np": 2, "expect_can_be_refined": False,
                          "source": "test/test_octree_merging.jl:274-290"},
    }


def scen_octree_sorting():
    # test/test_octree_sorting.jl
    def p(octant, v, w):
        return octant_particle(octant, v, w=w, x=(0.0, 0.0, 0.0))

    def create9(extra, reverse):
        rr = range(8, 0, -1) if reverse else range(1, 9)
        ps = []
        for octant in rr:
            ps.append(p(octant, 1.0, octant))
            if octant == extra:
                ps.append(p(octant, 2.0, octant))
        return ps

    def create7(missing, reverse):
        rr = range(8, 0, -1) if reverse else range(1, 9)
        return [p(o, 1.0, o) for o in rr if o != missing]

    def create15(wnest):
        mia = [12, 15, 2, 14, 13, 7, 8, 10, 5, 6, 1, 9, 4, 3, 11]
        vp = [None] * 15
        i = 0
        for vx in (-1.0, -3.0):
            for vy in (1.0, 3.0):
                for vz in (-3.0, -1.0):
                    vp[mia[i] - 1] = particle(wnest, (vx, vy, vz), (0, 0, 0))
                    i += 1
        for octant in range(8, 0, -1):
            if octant != 3:
                vp[mia[i] - 1] = p(octant, 1.0, 1.0)
                i += 1
        return vp

    conv = create9(3, False)[4:9] + create9(3, True)[5:9]
    return {
        "name": "octree_sorting",
        "source": "test/test_octree_sorting.jl",
        "octants": {"vmid": [-1.0, -1.0, -1.0],
                    "cases": [[[-2, -2, -2], 1], [[2, -2, -2], 2], [[-2, 2, -2], 3], [[2, 2, -2], 4],
                              [[-2, -2, 2], 5], [[2, -2, 2], 6], [[-2, 2, 2], 7], [[2, 2, 2], 8]],
                    "source": "test/test_octree_sorting.jl:114-139"},
        "nine_reverse": {"particles": create9(3, True), "expect_Nbins": 8,
                         "expect_pis": [9 - i + 1 for i in range(1, 10)],
                         "source": "test/test_octree_sorting.jl:141-160"},
        "nine_mixed": {"particles": conv, "expect_Nbins": 8, "expect_pis": [9, 8, 7, 6, 1, 2, 3, 4, 5],
                       "expect_bin_start": [1, 2, 3, 5, 6, 7, 8, 9], "expect_bin_end": [1, 2, 4, 5, 6, 7, 8, 9],
                       "expect_np": [1, 1, 2, 1, 1, 1, 1, 1], "expect_w": [1, 2, 6, 4, 5, 6, 7, 8],
                       "two_group_indexer": [9, 1, 3, 3, 4, 9, 6],
                       "source": "test/test_octree_sorting.jl:162-204"},
        "seven": {"particles": create7(5, True), "expect_Nbins": 7, "expect_pis": [7, 6, 5, 4, 3, 2, 1],
                  "expect_bin_start": [1, 2, 3, 4, 5, 6, 7], "expect_bin_end": [1, 2, 3, 4, 5, 6, 7],
                  "expect_np": [1] * 7, "expect_w": [1, 2, 3, 4, 6, 7, 8],
                  "source": "test/test_octree_sorting.jl:206-225"},
        "nested15": {"particles": create15(0.5), "init_bin_bounds": "MinMaxVelSym",
                     "first_split": {"expect_Nbins": 8, "expect_pis_1_2": [11, 3], "expect_bin3": [3, 10],
                                     "expect_sorted_3_10": [2, 7, 8, 10, 12, 13, 14, 15],
                                     "expect_pis_11_15": [4, 9, 1, 6, 5],
                                     "expect_np": [1, 1, 8, 1, 1, 1, 1, 1], "expect_w": [1, 1, 4.0, 1, 1, 1, 1, 1]},
                     "second_split": {"bin": 3, "expect_Nbins": 15,
                                      "expect_bin_start_1_3": [1, 2, 3],
                                      "expect_bin_start_4_8": [11, 12, 13, 14, 15],
                                      "expect_bin_start_9_15": [4, 5, 6, 7, 8, 9, 10],
                                      "expect_np": [1] * 15,
                                      "expect_w": [1, 1, 0.5, 1, 1, 1, 1, 1, 0.5, 0.5, 0.5, 0.5, 0.5, 0.5, 0.5]},
                     "source": "test/test_octree_sorting.jl:228-304"},
    }


def scen_octree_bounds():
    # test/test_octree_bounds_and_splitting.jl:25-137
    mia = [12, 15, 2, 14, 13, 7, 8, 10, 5, 6, 1, 9, 4, 3, 11]
    vp = [None] * 15
    i = 0
    for vx in (-1.0, -3.0):
        for vy in (1.0, 3.0):
            for vz in (-3.0, -1.0):
                vp[mia[i] - 1] = particle(1.0, (vx, vy, vz), (0, 0, 0))
                i += 1
    for octant in range(8, 0, -1):
        if octant != 3:
            vp[mia[i] - 1] = octant_particle(octant, 1.0, w=1.0, x=(0, 0, 0))
            i += 1
    eight = [octant_particle(o, 1.0, w=1.0, x=(0, 0, 0), v0=(1.0, 1.0, 1.0)) for o in range(1, 9)]
    return {
        "name": "octree_bounds",
        "source": "test/test_octree_bounds_and_splitting.jl:79-137",
        "eight": eight,
        "c_bounds": 299792458.0,
        "fifteen": vp,
        "sym_vmax": [3.0, 3.0, 3.0],
        "minmax_vmin": [-3.0, -1.0, -3.0],
        "minmax_vmax": [1.0, 3.0, 1.0],
        "outlier_v": [120000.0, -440000.0, 920000.0],
    }


def scen_computes():
    # test/test_computes.jl:6-41, 83-113
    return {
        "name": "computes_uniform",
        "source": "test/test_computes.jl:6-41,83-113",
        "n_particles": 2000, "n_dens": 1e25, "v0": [-1.0, 2.0, -4.0], "x0": [10.0, 20.0, 30.0],
        "tol_small": 1e-8,
        "avg": {"T": [100.0, 200.0], "n": [2e11, 4e11], "np": [100, 200], "v": [1e3, 2e3],
                "expect": {"T": 150.0, "n": 3e11, "np": 150.0, "v": 1.5e3}, "tol": "2eps"},
    }


def main():
    data = {
        "about": "Known-answer vectors transcribed from Merzbild.jl v0.7.10 test/ (see each 'source').",
        "species": {"Ar": {"mass": AR_MASS}, "He": {"mass": HE_MASS}},
        "vhs": {"Ar,Ar": [4.11e-10, 0.81, 273.0], "Ar,He": [3.25e-10, 0.735, 273.0], "He,He": [2.33e-10, 0.66, 273.0]},
        "pseudo_maxwell": {"Ar,Ar": [4.11e-10, 1.0, 273.0], "Ar,He": [3.25e-10, 1.0, 273.0],
                           "He,He": [2.33e-10, 1.0, 273.0]},
        "data_source": "data/particles.toml, data/vhs.toml, data/pseudo_maxwell.toml; asserted in test/runtests.jl:85-102",
        "scenarios": [scen_grid_sorting(), scen_convection(), scen_convection_noncontiguous(), scen_collision_utils(),
                      scen_octree_merge(), scen_octree_sorting(), scen_octree_bounds(), scen_computes()],
    }
    path = os.path.join(HERE, "reference_kat.json")
    with open(path, "w") as f:
        json.dump(data, f, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main()
