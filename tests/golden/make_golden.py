"""Generates the golden fixtures in tests/golden/ from the UNMODIFIED reference.

Builds oracle/_ref/refgen with oracle/build_ref.sh (it compiles the reference
sources XPBDFEM/{Fem,Geo,Connectivity,Allocator,MeshGen,vectormath,DebugGeo}.cpp
where they lie, plus the harness driver oracle/refgen.cpp), runs it for every
case in CASES, and stores each case's arrays as <name>.npz next to a
manifest.json with the parameters. Needs the reference tree, so it runs in the
development container only; the fixtures are committed and the tests read
them without the reference.

    python tests/golden/make_golden.py            # every case
    python tests/golden/make_golden.py NAME ...   # only these cases (the
                                                  # manifest keeps the others)
"""
import json
import os
import struct
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REFGEN = os.path.join(ROOT, "oracle", "_ref", "refgen")
sys.path.insert(0, os.path.join(ROOT, "oracle"))

DT = 1.0 / 1200.0
# compliance = 4 (1 + nu) / E for the Neo-Hookean cases (mu_ref = mu / 2).
C1_COMPLIANCE = 4.0 * 1.5 / 1e5

CASES = [
    ("meshgen_8x2x2", ["meshgen", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0]),
    ("meshgen_3x2x2_mirror_wonky", ["meshgen", 3, 2, 2, 0.1, 0.1, 0.1, 1, 0.3]),
    ("meshgen_4x3x2_aniso_wonky", ["meshgen", 4, 3, 2, 0.1, 0.05, 0.07, 0, 0.5]),
    ("init_8x2x2", ["init", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0]),
    ("init_3x2x2_mirror_wonky", ["init", 3, 2, 2, 0.1, 0.1, 0.1, 1, 0.3, 1000.0]),
    ("init_5x3x2_aniso_wonky", ["init", 5, 3, 2, 0.02, 0.03, 0.04, 0, 0.4, 500.0]),
    ("solve_nh_sim_incompressible", ["solve", 11, 64, 4, 1, C1_COMPLIANCE, 0.5, DT]),
    ("solve_nh_sim_nu045", ["solve", 12, 64, 4, 1, 0.01, 0.45, DT]),
    ("solve_yeoh_sim_incompressible", ["solve", 13, 64, 7, 1, 3.2, 0.5, DT]),
    ("solve_nh_serial_nu045", ["solve", 14, 64, 4, 0, 0.01, 0.45, DT]),
    ("solve_yeoh_serial_nu049", ["solve", 15, 64, 7, 0, 0.5, 0.49, DT]),
    ("substep_c1_nh_native", ["substep", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 4, 1, C1_COMPLIANCE, 0.5,
                              0.0, -9.81, DT, 40, 1]),
    ("substep_c1_yeoh_native", ["substep", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 7, 1, 3.2e-4, 0.5,
                                0.0, -9.81, DT, 40, 1]),
    ("substep_wonky_nh_serial_native", ["substep", 4, 3, 2, 0.05, 0.05, 0.05, 0.3, 1000.0, 4, 0, 1e-3, 0.45,
                                        -2.0, -9.81, DT, 10, 1]),
    ("ordered_c1_nh_star", ["ordered", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 4, 1, C1_COMPLIANCE, 0.5,
                            0.0, -9.81, DT, 40, 1]),
    ("ordered_c1_yeoh_tet", ["ordered", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 7, 1, 3.2e-4, 0.5,
                             0.0, -9.81, DT, 40, 1]),
    # the small cantilever configuration over its full 100 frames (20
    # substeps of 1/1200 s each), in the GPU's colour order
    ("ordered_c1_nh_100frames_star", ["ordered", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 4, 1, C1_COMPLIANCE, 0.5,
                                      0.0, -9.81, DT, 2000, 1]),
    ("ordered_c1_yeoh_100frames_star", ["ordered", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 7, 1, 3.2e-4, 0.5,
                                        0.0, -9.81, DT, 2000, 1]),
    # compressible (nu < 0.5): the coupled solve is well conditioned here, so
    # an FP32 implementation can be held to 1e-5 of the reference's own path
    ("ordered_c1_nh_nu045_star", ["ordered", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 4, 1, 4.0 * 1.45 / 1e5, 0.45,
                                  0.0, -9.81, DT, 40, 1]),
    ("ordered_c1_yeoh_nu049_tet", ["ordered", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 7, 1, 3.2e-4, 0.49,
                                   0.0, -9.81, DT, 40, 1]),
    ("ordered_wonky_nh_serial_nu045_star", ["ordered", 4, 3, 2, 0.05, 0.05, 0.05, 0.3, 1000.0, 4, 0, 1e-3, 0.45,
                                            -2.0, -9.81, DT, 10, 1]),
    # damping (GeoLinear3d::Damp and the in-solve Rayleigh terms): trailing
    # args damping, pbdDamping, drag, Rayleigh type (0 Paper, 1 Limit, 2 Post,
    # 3 PostAmortized), spacing (the demo's kSpacing)
    ("damped_c1_nh_nu045_amortized_pbd_star", ["damped", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 4, 1, 4.0 * 1.45 / 1e5,
                                               0.45, 0.0, -9.81, DT, 40, 1, 0.01, 0.03, 0.002, 3, 0.1]),
    ("damped_c1_nh_nu045_post_star", ["damped", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 4, 1, 4.0 * 1.45 / 1e5, 0.45,
                                      0.0, -9.81, DT, 40, 1, 0.01, 0.0, 0.0, 2, 0.1]),
    ("damped_c1_nh_nu045_paper_star", ["damped", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 4, 1, 4.0 * 1.45 / 1e5, 0.45,
                                       0.0, -9.81, DT, 40, 1, 0.01, 0.0, 0.0, 0, 0.1]),
    ("damped_c1_nh_nu045_limit_star", ["damped", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 4, 1, 4.0 * 1.45 / 1e5, 0.45,
                                       0.0, -9.81, DT, 40, 1, 0.01, 0.0, 0.0, 1, 0.1]),
    ("damped_c1_yeoh_nu049_amortized_pbd_tet", ["damped", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 7, 1, 3.2e-4, 0.49,
                                                0.0, -9.81, DT, 40, 1, 0.02, 0.05, 0.0, 3, 0.1]),
    ("damped_wonky_nh_serial_post_pbd_star", ["damped", 4, 3, 2, 0.05, 0.05, 0.05, 0.3, 1000.0, 4, 0, 1e-3, 0.45,
                                              -2.0, -9.81, DT, 10, 1, 0.01, 0.05, 0.0, 2, 0.05]),
    ("damped_wonky_nh_serial_limit_pbd_star", ["damped", 4, 3, 2, 0.05, 0.05, 0.05, 0.3, 1000.0, 4, 0, 1e-3, 0.45,
                                               -2.0, -9.81, DT, 10, 1, 0.01, 0.05, 0.0, 1, 0.05]),
    # the other energy models of SolveElement on linear tets (XPBDFEM/Fem.cpp:
    # 872-888): Pixar (0), PixarReduced (1), PixarSel (2), Mixed (3), YeohSkin
    # (5), YeohSkinSel (6), the cube models (11: no-op on tets), an id above
    # 12 (MixedSel)
    ("solve_pixar_nu045", ["solve", 21, 64, 0, 1, 0.01, 0.45, DT]),
    ("solve_pixar_reduced_nu040", ["solve", 22, 64, 1, 0, 0.02, 0.40, DT]),
    ("solve_pixarsel_nu049", ["solve", 23, 64, 2, 1, 0.01, 0.49, DT]),
    ("solve_mixed_sim_nu045", ["solve", 24, 64, 3, 1, 0.01, 0.45, DT]),
    ("solve_mixed_sim_incompressible", ["solve", 25, 64, 3, 1, C1_COMPLIANCE, 0.5, DT]),
    ("solve_mixed_serial_nu049", ["solve", 26, 64, 3, 0, 0.01, 0.49, DT]),
    ("solve_yeohskin_sim_nu045", ["solve", 27, 64, 5, 1, 0.5, 0.45, DT]),
    ("solve_yeohskin_sim_incompressible", ["solve", 28, 64, 5, 1, 3.2, 0.5, DT]),
    ("solve_yeohskinsel_serial_nu049", ["solve", 29, 64, 6, 0, 0.5, 0.49, DT]),
    ("solve_cube_neo_noop", ["solve", 30, 16, 11, 1, 0.01, 0.45, DT]),
    ("solve_id20_mixedsel", ["solve", 31, 64, 20, 1, 0.01, 0.45, DT]),
    # whole substeps in the GPU's colour order with those models (the `damped`
    # command, damping 0 where none is wanted); trailing arg: volume passes
    ("model_c1_pixar_nu045_star", ["damped", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 0, 1, 4.0 * 1.45 / 1e5, 0.45,
                                   0.0, -9.81, DT, 40, 1, 0.0, 0.0, 0.0, 2, 0.1]),
    ("model_c1_pixarsel_nu045_tet", ["damped", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 2, 1, 4.0 * 1.45 / 1e5, 0.45,
                                     0.0, -9.81, DT, 40, 1, 0.0, 0.0, 0.0, 2, 0.1]),
    ("model_c1_mixed_nu045_star", ["damped", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 3, 1, 4.0 * 1.45 / 1e5, 0.45,
                                   0.0, -9.81, DT, 40, 1, 0.0, 0.0, 0.0, 2, 0.1]),
    ("model_wonky_mixed_serial_nu045_star", ["damped", 4, 3, 2, 0.05, 0.05, 0.05, 0.3, 1000.0, 3, 0, 1e-3, 0.45,
                                             -2.0, -9.81, DT, 10, 1, 0.0, 0.0, 0.0, 2, 0.05]),
    ("model_c1_yeohskin_nu049_tet", ["damped", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 5, 1, 3.2e-4, 0.49,
                                     0.0, -9.81, DT, 40, 1, 0.0, 0.0, 0.0, 2, 0.1]),
    ("model_wonky_yeohskinsel_serial_nu049_star", ["damped", 4, 3, 2, 0.05, 0.05, 0.05, 0.3, 1000.0, 6, 0, 0.5,
                                                   0.49, -2.0, -9.81, DT, 10, 1, 0.0, 0.0, 0.0, 2, 0.05]),
    ("model_c1_cube_pbd_star", ["damped", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 11, 1, 4.0 * 1.45 / 1e5, 0.45,
                                0.0, -9.81, DT, 20, 1, 0.01, 0.03, 0.0, 2, 0.1]),
    ("model_c1_pixar_amortized_pbd_star", ["damped", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 0, 1, 4.0 * 1.45 / 1e5,
                                           0.45, 0.0, -9.81, DT, 40, 1, 0.01, 0.03, 0.002, 3, 0.1]),
    ("model_c1_pixar_paper_tet", ["damped", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 0, 1, 4.0 * 1.45 / 1e5, 0.45,
                                  0.0, -9.81, DT, 40, 1, 0.01, 0.0, 0.0, 0, 0.1]),
    ("model_c1_mixed_limit_star", ["damped", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 3, 1, 4.0 * 1.45 / 1e5, 0.45,
                                   0.0, -9.81, DT, 40, 1, 0.01, 0.0, 0.0, 1, 0.1]),
    ("model_wonky_yeohskin_serial_post_star", ["damped", 4, 3, 2, 0.05, 0.05, 0.05, 0.3, 1000.0, 5, 0, 0.5, 0.45,
                                               -2.0, -9.81, DT, 10, 1, 0.01, 0.0, 0.0, 2, 0.05]),
    ("volume_c1_nh_nu045_2_star", ["damped", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 4, 1, 4.0 * 1.45 / 1e5, 0.45,
                                   0.0, -9.81, DT, 40, 1, 0.0, 0.0, 0.0, 2, 0.1, 2]),
    ("volume_c1_yeoh_nu049_3_tet", ["damped", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 7, 1, 3.2e-4, 0.49,
                                    0.0, -9.81, DT, 40, 1, 0.0, 0.0, 0.0, 2, 0.1, 3]),
    ("volume_wonky_pixar_1_post_pbd_star", ["damped", 4, 3, 2, 0.05, 0.05, 0.05, 0.3, 1000.0, 0, 1, 1e-3, 0.45,
                                            -2.0, -9.81, DT, 10, 1, 0.01, 0.05, 0.0, 2, 0.05, 1]),
    # continuous-pressure models (one constraint pair per vertex one-ring,
    # XPBDFEM/Geo.cpp:147-193): the `damped` arguments, with the vertex ring
    # order of the GPU schedule (and the tet order for the PBD damping)
    ("rings_c1_cpixar_nu045_star", ["rings", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 8, 1, 4.0 * 1.45 / 1e5, 0.45,
                                    0.0, -9.81, DT, 40, 1, 0.0, 0.0, 0.0, 2, 0.1]),
    ("rings_c1_cmixed_nu045_star", ["rings", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 9, 1, 4.0 * 1.45 / 1e5, 0.45,
                                    0.0, -9.81, DT, 40, 1, 0.0, 0.0, 0.0, 2, 0.1]),
    ("rings_c1_cmixed_incompressible_star", ["rings", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 9, 1, C1_COMPLIANCE, 0.5,
                                             0.0, -9.81, DT, 40, 1, 0.0, 0.0, 0.0, 2, 0.1]),
    ("rings_c1_cskin_nu049_star", ["rings", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 10, 1, 3.2e-4, 0.49,
                                   0.0, -9.81, DT, 40, 1, 0.0, 0.0, 0.0, 2, 0.1]),
    ("rings_wonky_cmixed_paper_star", ["rings", 4, 3, 2, 0.05, 0.05, 0.05, 0.3, 1000.0, 9, 1, 1e-3, 0.45,
                                       -2.0, -9.81, DT, 10, 1, 0.01, 0.0, 0.0, 0, 0.05]),
    ("rings_c1_cskin_limit_star", ["rings", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 10, 1, 3.2e-4, 0.45,
                                   0.0, -9.81, DT, 40, 1, 0.01, 0.0, 0.0, 1, 0.1]),
    ("rings_c1_cmixed_amortized_pbd_star", ["rings", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 9, 1, 4.0 * 1.45 / 1e5,
                                            0.45, 0.0, -9.81, DT, 40, 1, 0.01, 0.03, 0.002, 3, 0.1]),
    ("rings_wonky_cpixar_post_star", ["rings", 4, 3, 2, 0.05, 0.05, 0.05, 0.3, 1000.0, 8, 1, 1e-3, 0.45,
                                      -2.0, -9.81, DT, 10, 1, 0.01, 0.0, 0.0, 2, 0.05]),
    # the Right lock (Settings_LockRight, XPBDFEM/Geo.cpp:323-331): the
    # `damped` arguments with volumePasses, then lockedRightTransform3d
    # (column-major; the demo's rotation(0.3) * scale(1.2, 1) form,
    # XPBDFEM/Demo.cpp:71-79) and Geo3d::origin
    ("locked_c1_nh_nu045_star", ["locked", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 4, 1, 4.0 * 1.45 / 1e5, 0.45,
                                 0.0, -9.81, DT, 40, 1, 0.0, 0.0, 0.0, 2, 0.1, 0,
                                 1.1464038, 0.35462425, 0.0, -0.29552021, 0.9553365, 0.0, 0.0, 0.0, 1.0,
                                 0.02, -0.01, 0.005]),
    ("locked_c1_yeoh_nu049_amortized_pbd_tet", ["locked", 8, 2, 2, 0.1, 0.1, 0.1, 0.0, 1000.0, 7, 1, 3.2e-4, 0.49,
                                                0.0, -9.81, DT, 40, 1, 0.02, 0.05, 0.0, 3, 0.1, 0,
                                                1.1464038, 0.35462425, 0.0, -0.29552021, 0.9553365, 0.0, 0.0, 0.0,
                                                1.0, 0.0, 0.0, 0.0]),
    ("locked_wonky_nh_serial_nu045_right_only_star", ["locked", 4, 3, 2, 0.05, 0.05, 0.05, 0.3, 1000.0, 4, 0, 1e-3,
                                                      0.45, -2.0, -9.81, DT, 10, 0, 0.0, 0.0, 0.0, 2, 0.05, 0,
                                                      1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0, 0.01, 0.02, -0.03]),
    # linear hexahedra (GeoLinear3d's hex loops on a GenerateHexBlock mesh):
    # the `h` commands take the element pattern after the scale; the substep
    # cases run in the GPU's hex colour order
    ("hmeshgen_3x2x2_mirror_wonky", ["hmeshgen", 3, 2, 2, 0.1, 0.1, 0.1, 1, 0.3]),
    ("hinit_4x2x2", ["hinit", 4, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0]),
    ("hinit_3x2x2_mirror_wonky", ["hinit", 3, 2, 2, 0.1, 0.1, 0.1, 1, 0.3, 1000.0]),
    ("hinit_4x3x2_aniso_wonky", ["hinit", 4, 3, 2, 0.02, 0.03, 0.04, 0, 0.4, 500.0]),
    ("hsolve_nh_sim_nu045", ["hsolve", 41, 32, 4, 1, 0.01, 0.45, DT]),
    ("hsolve_nh_sim_incompressible", ["hsolve", 42, 32, 4, 1, C1_COMPLIANCE, 0.5, DT]),
    ("hsolve_nh_serial_nu045", ["hsolve", 43, 32, 4, 0, 0.01, 0.45, DT]),
    ("hsolve_yeohfast_sim_nu049", ["hsolve", 44, 32, 7, 1, 0.5, 0.49, DT]),
    ("hsolve_yeohfast_serial_incompressible", ["hsolve", 45, 32, 7, 0, 3.2, 0.5, DT]),
    ("hsolve_mixed_sim_nu045", ["hsolve", 46, 32, 3, 1, 0.01, 0.45, DT]),
    ("hsolve_mixed_serial_nu049", ["hsolve", 47, 32, 3, 0, 0.01, 0.49, DT]),
    ("hsolve_yeohskin_sim_nu045", ["hsolve", 48, 32, 5, 1, 0.5, 0.45, DT]),
    ("hsolve_yeohskinsel_sim_nu049", ["hsolve", 49, 32, 6, 1, 0.5, 0.49, DT]),
    ("hsolve_yeohskinsel_serial_nu045", ["hsolve", 50, 32, 6, 0, 0.5, 0.45, DT]),
    ("hsolve_pixar_nu045", ["hsolve", 51, 32, 0, 1, 0.01, 0.45, DT]),
    ("hsolve_pixar_reduced_nu040", ["hsolve", 52, 32, 1, 0, 0.02, 0.40, DT]),
    ("hsolve_pixarsel_nu049", ["hsolve", 53, 32, 2, 1, 0.01, 0.49, DT]),
    ("hsolve_id20_mixedsel", ["hsolve", 54, 32, 20, 1, 0.01, 0.45, DT]),
    ("hsolve_cube_neo_fast", ["hsolve", 55, 32, 11, 1, C1_COMPLIANCE, 0.5, DT]),
    ("hsolve_cube_neo_nu045", ["hsolve", 56, 32, 11, 1, 0.01, 0.45, DT]),
    ("hsolve_cube_skin_nu049", ["hsolve", 57, 32, 12, 0, 0.5, 0.49, DT]),
    ("hsolve_cube_skin_incompressible", ["hsolve", 58, 32, 12, 1, 3.2, 0.5, DT]),
    ("hordered_c1_nh_nu045", ["hordered", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 4, 1, 4.0 * 1.45 / 1e5, 0.45,
                              0.0, -9.81, DT, 40, 1]),
    ("hordered_c1_nh_incompressible", ["hordered", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 4, 1, C1_COMPLIANCE, 0.5,
                                       0.0, -9.81, DT, 40, 1]),
    ("hordered_c1_yeohfast_nu049", ["hordered", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 7, 1, 3.2e-4, 0.49,
                                    0.0, -9.81, DT, 40, 1]),
    ("hordered_wonky_nh_serial_nu045", ["hordered", 4, 3, 2, 0.05, 0.05, 0.05, 1, 0.3, 1000.0, 4, 0, 1e-3, 0.45,
                                        -2.0, -9.81, DT, 10, 1]),
    ("hordered_c1_mixed_nu045", ["hordered", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 3, 1, 4.0 * 1.45 / 1e5, 0.45,
                                 0.0, -9.81, DT, 40, 1]),
    ("hordered_wonky_yeohskinsel_serial_nu049", ["hordered", 4, 3, 2, 0.05, 0.05, 0.05, 1, 0.3, 1000.0, 6, 0, 0.5,
                                                 0.49, -2.0, -9.81, DT, 10, 1]),
    ("hordered_c1_pixar_nu045", ["hordered", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 0, 1, 4.0 * 1.45 / 1e5, 0.45,
                                 0.0, -9.81, DT, 40, 1]),
    ("hdamped_c1_nh_nu045_post_pbd", ["hdamped", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 4, 1, 4.0 * 1.45 / 1e5, 0.45,
                                      0.0, -9.81, DT, 40, 1, 0.01, 0.03, 0.0, 2, 0.1]),
    ("hdamped_c1_nh_nu045_amortized_pbd", ["hdamped", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 4, 1, 4.0 * 1.45 / 1e5,
                                           0.45, 0.0, -9.81, DT, 40, 1, 0.01, 0.03, 0.002, 3, 0.1]),
    ("hdamped_c1_nh_nu045_paper", ["hdamped", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 4, 1, 4.0 * 1.45 / 1e5, 0.45,
                                   0.0, -9.81, DT, 40, 1, 0.01, 0.0, 0.0, 0, 0.1]),
    ("hdamped_c1_nh_nu045_limit", ["hdamped", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 4, 1, 4.0 * 1.45 / 1e5, 0.45,
                                   0.0, -9.81, DT, 40, 1, 0.01, 0.0, 0.0, 1, 0.1]),
    ("hdamped_wonky_yeohskin_serial_post", ["hdamped", 4, 3, 2, 0.05, 0.05, 0.05, 1, 0.3, 1000.0, 5, 0, 0.5, 0.45,
                                            -2.0, -9.81, DT, 10, 1, 0.01, 0.0, 0.0, 2, 0.05]),
    ("hvolume_c1_nh_nu045_2", ["hdamped", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 4, 1, 4.0 * 1.45 / 1e5, 0.45,
                               0.0, -9.81, DT, 40, 1, 0.0, 0.0, 0.0, 2, 0.1, 2]),
    ("hordered_c1_cube_neo_fast", ["hordered", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 11, 1, C1_COMPLIANCE, 0.5,
                                   0.0, -9.81, DT, 40, 1]),
    ("hordered_wonky_cube_neo_nu045", ["hordered", 4, 3, 2, 0.05, 0.05, 0.05, 1, 0.3, 1000.0, 11, 1, 1e-3, 0.45,
                                       -2.0, -9.81, DT, 10, 1]),
    ("hordered_c1_cube_skin_nu049", ["hordered", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 12, 1, 3.2e-4, 0.49,
                                     0.0, -9.81, DT, 40, 1]),
    ("hdamped_c1_cube_neo_nu045_paper", ["hdamped", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 11, 1, 4.0 * 1.45 / 1e5,
                                         0.45, 0.0, -9.81, DT, 40, 1, 0.01, 0.0, 0.0, 0, 0.1]),
    ("hdamped_c1_cube_skin_nu045_limit", ["hdamped", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 12, 1, 3.2e-4, 0.45,
                                          0.0, -9.81, DT, 40, 1, 0.01, 0.0, 0.0, 1, 0.1]),
    ("hdamped_c1_cube_neo_incompressible_amortized_pbd", ["hdamped", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 11, 1,
                                                          C1_COMPLIANCE, 0.5, 0.0, -9.81, DT, 40, 1, 0.01, 0.03,
                                                          0.002, 3, 0.1, 1]),
    # continuous-pressure models on a hex mesh (SolveRing's hex branch,
    # XPBDFEM/Geo.cpp:147-225; XPBDFEM/Fem.cpp:983-1036): the `damped`
    # arguments with the pattern after the scale; stdin holds the GPU's hex
    # colour order (PBD damping) and its ring vertex order
    ("hrings_c1_cpixar_nu045", ["hrings", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 8, 1, 4.0 * 1.45 / 1e5, 0.45,
                                0.0, -9.81, DT, 40, 1, 0.0, 0.0, 0.0, 2, 0.1]),
    ("hrings_c1_cmixed_nu045", ["hrings", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 9, 1, 4.0 * 1.45 / 1e5, 0.45,
                                0.0, -9.81, DT, 40, 1, 0.0, 0.0, 0.0, 2, 0.1]),
    ("hrings_c1_cmixed_incompressible", ["hrings", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 9, 1, C1_COMPLIANCE, 0.5,
                                         0.0, -9.81, DT, 40, 1, 0.0, 0.0, 0.0, 2, 0.1]),
    ("hrings_c1_cskin_nu049", ["hrings", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 10, 1, 3.2e-4, 0.49,
                               0.0, -9.81, DT, 40, 1, 0.0, 0.0, 0.0, 2, 0.1]),
    ("hrings_wonky_cmixed_paper", ["hrings", 4, 3, 2, 0.05, 0.05, 0.05, 1, 0.3, 1000.0, 9, 1, 1e-3, 0.45,
                                   -2.0, -9.81, DT, 10, 1, 0.01, 0.0, 0.0, 0, 0.05]),
    ("hrings_c1_cskin_limit", ["hrings", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 10, 1, 3.2e-4, 0.45,
                               0.0, -9.81, DT, 40, 1, 0.01, 0.0, 0.0, 1, 0.1]),
    ("hrings_c1_cmixed_amortized_pbd", ["hrings", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 9, 1, 4.0 * 1.45 / 1e5,
                                        0.45, 0.0, -9.81, DT, 40, 1, 0.01, 0.03, 0.002, 3, 0.1]),
    ("hrings_wonky_cpixar_post", ["hrings", 4, 3, 2, 0.05, 0.05, 0.05, 1, 0.3, 1000.0, 8, 1, 1e-3, 0.45,
                                  -2.0, -9.81, DT, 10, 1, 0.01, 0.0, 0.0, 2, 0.05]),
    # quadratic tets (GeoQuadratic3d on a GenerateTetBlock mesh; element
    # type T10 in the settings' flags): the `q` commands take the pattern
    # after the scale; the substep cases run in the GPU's T10 colour order
    ("qinit_3x2x2", ["qinit", 3, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0]),
    ("qinit_3x2x2_mirror_wonky", ["qinit", 3, 2, 2, 0.1, 0.1, 0.1, 1, 0.3, 1000.0]),
    ("qsolve_nh_sim_nu045", ["qsolve", 61, 32, 4, 1, 0.01, 0.45, DT]),
    ("qsolve_nh_sim_incompressible", ["qsolve", 62, 32, 4, 1, C1_COMPLIANCE, 0.5, DT]),
    ("qsolve_nh_serial_nu045", ["qsolve", 63, 32, 4, 0, 0.01, 0.45, DT]),
    ("qsolve_yeohfast_sim_nu049", ["qsolve", 64, 32, 7, 1, 0.5, 0.49, DT]),
    ("qsolve_mixed_sim_nu045", ["qsolve", 65, 32, 3, 1, 0.01, 0.45, DT]),
    ("qsolve_yeohskinsel_serial_nu045", ["qsolve", 66, 32, 6, 0, 0.5, 0.45, DT]),
    ("qsolve_pixar_nu045", ["qsolve", 67, 32, 0, 1, 0.01, 0.45, DT]),
    ("qsolve_pixarsel_nu049", ["qsolve", 68, 32, 2, 1, 0.01, 0.49, DT]),
    ("qordered_c1_nh_nu045", ["qordered", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 4, 1, 4.0 * 1.45 / 1e5, 0.45,
                              0.0, -9.81, DT, 40, 1]),
    ("qordered_c1_nh_incompressible", ["qordered", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 4, 1, C1_COMPLIANCE, 0.5,
                                       0.0, -9.81, DT, 40, 1]),
    ("qordered_wonky_yeohfast_serial_nu049", ["qordered", 4, 3, 2, 0.05, 0.05, 0.05, 1, 0.3, 1000.0, 7, 0, 3.2e-4,
                                              0.49, -2.0, -9.81, DT, 10, 1]),
    ("qordered_c1_mixed_nu045", ["qordered", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 3, 1, 4.0 * 1.45 / 1e5, 0.45,
                                 0.0, -9.81, DT, 40, 1]),
    ("qdamped_c1_nh_nu045_amortized_pbd", ["qdamped", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 4, 1, 4.0 * 1.45 / 1e5,
                                           0.45, 0.0, -9.81, DT, 40, 1, 0.01, 0.03, 0.002, 3, 0.1]),
    ("qdamped_c1_pixar_nu045_limit", ["qdamped", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 0, 1, 4.0 * 1.45 / 1e5,
                                      0.45, 0.0, -9.81, DT, 40, 1, 0.01, 0.0, 0.0, 1, 0.1]),
    ("qvolume_wonky_nh_serial_1_post", ["qdamped", 4, 3, 2, 0.05, 0.05, 0.05, 1, 0.3, 1000.0, 4, 0, 1e-3, 0.45,
                                        -2.0, -9.81, DT, 10, 1, 0.01, 0.0, 0.0, 2, 0.05, 1]),
    # continuous-pressure models on quadratic tets (SolveRing over the T10s
    # around each mesh vertex, XPBDFEM/Geo.cpp:147-225, 944-953, 971-1008):
    # the `qdamped` arguments; stdin holds the GPU's T10 colour order (PBD
    # damping) and its ring order over the mesh's own vertices
    ("qrings_c1_cpixar_nu045", ["qrings", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 8, 1, 4.0 * 1.45 / 1e5, 0.45,
                                0.0, -9.81, DT, 40, 1, 0.0, 0.0, 0.0, 2, 0.1]),
    ("qrings_c1_cmixed_nu045", ["qrings", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 9, 1, 4.0 * 1.45 / 1e5, 0.45,
                                0.0, -9.81, DT, 40, 1, 0.0, 0.0, 0.0, 2, 0.1]),
    ("qrings_c1_cmixed_incompressible", ["qrings", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 9, 1, C1_COMPLIANCE, 0.5,
                                         0.0, -9.81, DT, 40, 1, 0.0, 0.0, 0.0, 2, 0.1]),
    ("qrings_c1_cskin_nu049", ["qrings", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 10, 1, 3.2e-4, 0.49,
                               0.0, -9.81, DT, 40, 1, 0.0, 0.0, 0.0, 2, 0.1]),
    ("qrings_wonky_cmixed_paper", ["qrings", 4, 3, 2, 0.05, 0.05, 0.05, 1, 0.3, 1000.0, 9, 1, 1e-3, 0.45,
                                   -2.0, -9.81, DT, 10, 1, 0.01, 0.0, 0.0, 0, 0.05]),
    ("qrings_c1_cskin_limit", ["qrings", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 10, 1, 3.2e-4, 0.45,
                               0.0, -9.81, DT, 40, 1, 0.01, 0.0, 0.0, 1, 0.1]),
    ("qrings_c1_cmixed_amortized_pbd", ["qrings", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 9, 1, 4.0 * 1.45 / 1e5,
                                        0.45, 0.0, -9.81, DT, 40, 1, 0.01, 0.03, 0.002, 3, 0.1]),
    ("qrings_wonky_cpixar_post", ["qrings", 4, 3, 2, 0.05, 0.05, 0.05, 1, 0.3, 1000.0, 8, 1, 1e-3, 0.45,
                                  -2.0, -9.81, DT, 10, 1, 0.01, 0.0, 0.0, 2, 0.05]),
    ("hvolume_wonky_pixar_1_post_pbd", ["hdamped", 4, 3, 2, 0.05, 0.05, 0.05, 1, 0.3, 1000.0, 0, 1, 1e-3, 0.45,
                                        -2.0, -9.81, DT, 10, 1, 0.01, 0.05, 0.0, 2, 0.05, 1]),
    # quadratic hexahedra (GeoQuadratic3d on a GenerateHexBlock mesh, element
    # type H27): the `Q` commands; the substep cases run in the GPU's H27
    # colour order
    ("h27init_2x2x1", ["Qinit", 2, 2, 1, 0.1, 0.1, 0.1, 0, 0.0, 1000.0]),
    ("h27init_3x2x2_mirror_wonky", ["Qinit", 3, 2, 2, 0.1, 0.1, 0.1, 1, 0.3, 1000.0]),
    ("h27solve_nh_sim_nu045", ["Qsolve", 71, 16, 4, 1, 0.01, 0.45, DT]),
    ("h27solve_nh_sim_incompressible", ["Qsolve", 72, 16, 4, 1, C1_COMPLIANCE, 0.5, DT]),
    ("h27solve_nh_serial_nu045", ["Qsolve", 73, 16, 4, 0, 0.01, 0.45, DT]),
    ("h27solve_yeohfast_sim_nu049", ["Qsolve", 74, 16, 7, 1, 0.5, 0.49, DT]),
    ("h27solve_mixed_sim_nu045", ["Qsolve", 75, 16, 3, 1, 0.01, 0.45, DT]),
    ("h27solve_yeohskinsel_serial_nu045", ["Qsolve", 76, 16, 6, 0, 0.5, 0.45, DT]),
    ("h27solve_pixar_nu045", ["Qsolve", 77, 16, 0, 1, 0.01, 0.45, DT]),
    ("h27solve_pixarsel_nu049", ["Qsolve", 78, 16, 2, 1, 0.01, 0.49, DT]),
    ("h27ordered_c1_nh_nu045", ["Qordered", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 4, 1, 4.0 * 1.45 / 1e5, 0.45,
                                0.0, -9.81, DT, 20, 1]),
    ("h27ordered_c1_nh_incompressible", ["Qordered", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 4, 1, C1_COMPLIANCE,
                                         0.5, 0.0, -9.81, DT, 20, 1]),
    ("h27ordered_wonky_yeohfast_serial_nu049", ["Qordered", 4, 3, 2, 0.05, 0.05, 0.05, 1, 0.3, 1000.0, 7, 0, 3.2e-4,
                                                0.49, -2.0, -9.81, DT, 10, 1]),
    ("h27ordered_c1_mixed_nu045", ["Qordered", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 3, 1, 4.0 * 1.45 / 1e5, 0.45,
                                   0.0, -9.81, DT, 20, 1]),
    ("h27damped_c1_nh_nu045_amortized_pbd", ["Qdamped", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 4, 1,
                                             4.0 * 1.45 / 1e5, 0.45, 0.0, -9.81, DT, 20, 1, 0.01, 0.03, 0.002, 3,
                                             0.1]),
    ("h27damped_c1_pixar_nu045_limit", ["Qdamped", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 0, 1, 4.0 * 1.45 / 1e5,
                                        0.45, 0.0, -9.81, DT, 20, 1, 0.01, 0.0, 0.0, 1, 0.1]),
    ("h27volume_wonky_nh_serial_1_post", ["Qdamped", 4, 3, 2, 0.05, 0.05, 0.05, 1, 0.3, 1000.0, 4, 0, 1e-3, 0.45,
                                          -2.0, -9.81, DT, 10, 1, 0.01, 0.0, 0.0, 2, 0.05, 1]),
    # continuous-pressure models on quadratic hexes (SolveRing over the H27s
    # around each mesh vertex): the `Qdamped` arguments; stdin holds the GPU's
    # H27 colour order (PBD damping) and its ring order over the mesh's own
    # vertices
    ("h27rings_c1_cpixar_nu045", ["Qrings", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 8, 1, 4.0 * 1.45 / 1e5, 0.45,
                                0.0, -9.81, DT, 20, 1, 0.0, 0.0, 0.0, 2, 0.1]),
    ("h27rings_c1_cmixed_nu045", ["Qrings", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 9, 1, 4.0 * 1.45 / 1e5, 0.45,
                                0.0, -9.81, DT, 20, 1, 0.0, 0.0, 0.0, 2, 0.1]),
    ("h27rings_c1_cmixed_incompressible", ["Qrings", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 9, 1, C1_COMPLIANCE, 0.5,
                                         0.0, -9.81, DT, 20, 1, 0.0, 0.0, 0.0, 2, 0.1]),
    ("h27rings_c1_cskin_nu049", ["Qrings", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 10, 1, 3.2e-4, 0.49,
                               0.0, -9.81, DT, 20, 1, 0.0, 0.0, 0.0, 2, 0.1]),
    ("h27rings_wonky_cmixed_paper", ["Qrings", 4, 3, 2, 0.05, 0.05, 0.05, 1, 0.3, 1000.0, 9, 1, 1e-3, 0.45,
                                   -2.0, -9.81, DT, 10, 1, 0.01, 0.0, 0.0, 0, 0.05]),
    ("h27rings_c1_cskin_limit", ["Qrings", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 10, 1, 3.2e-4, 0.45,
                               0.0, -9.81, DT, 20, 1, 0.01, 0.0, 0.0, 1, 0.1]),
    ("h27rings_c1_cmixed_amortized_pbd", ["Qrings", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, 1000.0, 9, 1, 4.0 * 1.45 / 1e5,
                                        0.45, 0.0, -9.81, DT, 20, 1, 0.01, 0.03, 0.002, 3, 0.1]),
    ("h27rings_wonky_cpixar_post", ["Qrings", 4, 3, 2, 0.05, 0.05, 0.05, 1, 0.3, 1000.0, 8, 1, 1e-3, 0.45,
                                  -2.0, -9.81, DT, 10, 1, 0.01, 0.0, 0.0, 2, 0.05]),
    # meshes mixing tets and hexes (GeoLinear3d on one tagged stream): a
    # GenerateHexBlock mesh whose `split` cells ("checker": x + y + z even,
    # "left": x < W / 2) are GenerateTetBlock's six tets; args W H D sx sy sz
    # pattern wonkiness split, then refgen's `mixed` arguments (density
    # energy simultaneous compliance poisson gx gy dt nsub lockleft damping
    # pbdDamping drag rayleighType spacing volumePasses); stdin holds the
    # mesh, the GPU's tet colour order and its hex colour order
    ("mixed_c1_nh_nu045_checker", ["mixed", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, "checker", 1000.0, 4, 1,
                                   4.0 * 1.45 / 1e5, 0.45, 0.0, -9.81, DT, 40, 1, 0.0, 0.0, 0.0, 2, 0.1, 0]),
    ("mixed_c1_nh_incompressible_left", ["mixed", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, "left", 1000.0, 4, 1,
                                         C1_COMPLIANCE, 0.5, 0.0, -9.81, DT, 40, 1, 0.0, 0.0, 0.0, 2, 0.1, 0]),
    ("mixed_wonky_yeohfast_serial_nu049_checker", ["mixed", 4, 3, 2, 0.05, 0.05, 0.05, 1, 0.3, "checker", 1000.0, 7, 0,
                                                   3.2e-4, 0.49, -2.0, -9.81, DT, 10, 1, 0.0, 0.0, 0.0, 2, 0.05, 0]),
    ("mixed_c1_pixar_nu045_amortized_pbd_checker", ["mixed", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, "checker", 1000.0, 0, 1,
                                                    4.0 * 1.45 / 1e5, 0.45, 0.0, -9.81, DT, 40, 1, 0.01, 0.03, 0.002,
                                                    3, 0.1, 0]),
    ("mixed_c1_mixed_nu045_limit_left", ["mixed", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, "left", 1000.0, 3, 1,
                                         4.0 * 1.45 / 1e5, 0.45, 0.0, -9.81, DT, 40, 1, 0.01, 0.0, 0.0, 1, 0.1, 0]),
    ("mixed_wonky_nh_paper_volume_checker", ["mixed", 4, 3, 2, 0.05, 0.05, 0.05, 1, 0.3, "checker", 1000.0, 4, 1,
                                             1e-3, 0.45, -2.0, -9.81, DT, 10, 1, 0.01, 0.0, 0.0, 0, 0.05, 1]),
    ("mixed_c1_cube_neo_nu045_post_checker", ["mixed", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, "checker", 1000.0, 11, 1,
                                              4.0 * 1.45 / 1e5, 0.45, 0.0, -9.81, DT, 40, 1, 0.01, 0.0, 0.0, 2, 0.1,
                                              0]),
    ("mixed_c1_yeohskin_nu045_post_pbd_left", ["mixed", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, "left", 1000.0, 5, 1, 0.5,
                                               0.45, 0.0, -9.81, DT, 40, 1, 0.01, 0.05, 0.0, 2, 0.1, 0]),
    # the same meshes as GeoQuadratic3d (T10s and H27s in one body): refgen's
    # `qmixed`, stdin the mesh, the GPU's T10 colour order and its H27 colour
    # order
    ("qmixed_c1_nh_nu045_checker", ["qmixed", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, "checker", 1000.0, 4, 1,
                                    4.0 * 1.45 / 1e5, 0.45, 0.0, -9.81, DT, 20, 1, 0.0, 0.0, 0.0, 2, 0.1, 0]),
    ("qmixed_c1_nh_incompressible_left", ["qmixed", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, "left", 1000.0, 4, 1,
                                          C1_COMPLIANCE, 0.5, 0.0, -9.81, DT, 20, 1, 0.0, 0.0, 0.0, 2, 0.1, 0]),
    ("qmixed_wonky_yeohfast_serial_nu049_checker", ["qmixed", 4, 3, 2, 0.05, 0.05, 0.05, 1, 0.3, "checker", 1000.0, 7,
                                                    0, 3.2e-4, 0.49, -2.0, -9.81, DT, 10, 1, 0.0, 0.0, 0.0, 2, 0.05, 0]),
    ("qmixed_c1_pixar_nu045_amortized_pbd_checker", ["qmixed", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, "checker", 1000.0, 0, 1,
                                                     4.0 * 1.45 / 1e5, 0.45, 0.0, -9.81, DT, 20, 1, 0.01, 0.03, 0.002,
                                                     3, 0.1, 0]),
    ("qmixed_c1_mixed_nu045_limit_left", ["qmixed", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, "left", 1000.0, 3, 1,
                                          4.0 * 1.45 / 1e5, 0.45, 0.0, -9.81, DT, 20, 1, 0.01, 0.0, 0.0, 1, 0.1, 0]),
    ("qmixed_wonky_nh_paper_volume_checker", ["qmixed", 4, 3, 2, 0.05, 0.05, 0.05, 1, 0.3, "checker", 1000.0, 4, 1,
                                              1e-3, 0.45, -2.0, -9.81, DT, 10, 1, 0.01, 0.0, 0.0, 0, 0.05, 1]),
    ("qmixed_c1_yeohskin_nu045_post_pbd_left", ["qmixed", 8, 2, 2, 0.1, 0.1, 0.1, 0, 0.0, "left", 1000.0, 5, 1, 0.5,
                                                0.45, 0.0, -9.81, DT, 20, 1, 0.01, 0.05, 0.0, 2, 0.1, 0]),
]

MIXED_SPLITS = {"checker": lambda x, y, z, W: (x + y + z) % 2 == 0, "left": lambda x, y, z, W: 2 * x < W}


def mixed_mesh(args):
    """The mesh of a `mixed` case: (nodes, idx)."""
    import oracle  # noqa: E402
    W, H, D, sx, sy, sz, pattern, wonk, split = args[1:10]
    f = MIXED_SPLITS[split]
    return oracle.mixed_block(W, H, D, (sx, sy, sz), pattern, wonk, lambda x, y, z: f(x, y, z, W))


def parse(blob):
    out, i = {}, 0
    dt = {"f": np.float32, "d": np.float64, "I": np.uint32, "B": np.uint8}
    while i < len(blob):
        (n,) = struct.unpack_from("<I", blob, i); i += 4
        name = blob[i:i + n].decode(); i += n
        kind = chr(blob[i]); i += 1
        (cnt,) = struct.unpack_from("<Q", blob, i); i += 8
        a = np.frombuffer(blob, dt[kind], cnt, i).copy()
        i += a.nbytes
        out[name] = a
    return out


def main():
    subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    only = set(sys.argv[1:])
    unknown = only - {n for n, _ in CASES}
    if unknown:
        sys.exit(f"unknown cases: {sorted(unknown)}")
    manifest = {}
    mpath = os.path.join(HERE, "manifest.json")
    if only and os.path.exists(mpath):
        with open(mpath) as f:
            manifest = json.load(f)
    for name, args in CASES:
        if only and name not in only:
            continue
        argv = [REFGEN] + [str(a) for a in args]
        stdin = None
        extra = {}
        if args[0] in ("hordered", "hdamped"):
            import oracle  # noqa: E402
            W, H, D, sx, sy, sz, pattern, wonk = args[1:9]
            nodes, idx = oracle.gen_hex_block(W, H, D, (sx, sy, sz), pattern, wonk)
            hexes, _ = oracle.parse_hexes(idx)
            sch = oracle.hex_schedule(nodes, hexes, morton=1)
            order = sch["hex_order"].astype(np.uint32)
            stdin = struct.pack("<I", order.size) + order.tobytes()
            extra = {"order": order, "colour_hex_begin": sch["colour_hex_begin"]}
        if args[0] == "hrings":
            import oracle  # noqa: E402
            W, H, D, sx, sy, sz, pattern, wonk = args[1:9]
            nodes, idx = oracle.gen_hex_block(W, H, D, (sx, sy, sz), pattern, wonk)
            hexes, _ = oracle.parse_hexes(idx)
            sch = oracle.hex_schedule(nodes, hexes, morton=1)
            order = sch["hex_order"].astype(np.uint32)
            rs = oracle.ring_schedule(nodes, hexes, morton=1)
            vorder = rs["vert_order"].astype(np.uint32)
            stdin = struct.pack("<I", order.size) + order.tobytes() + struct.pack("<I", vorder.size) + vorder.tobytes()
            extra = {"order": order, "colour_hex_begin": sch["colour_hex_begin"], "vorder": vorder,
                     "colour_vert_begin": rs["colour_vert_begin"]}
        if args[0] in ("Qordered", "Qdamped", "Qrings"):
            import oracle  # noqa: E402
            W, H, D, sx, sy, sz, pattern, wonk, dens = args[1:10]
            nodes, idx = oracle.gen_hex_block(W, H, D, (sx, sy, sz), pattern, wonk)
            q = oracle.QuadraticHex(nodes, idx, dens)
            sch = q.schedule(morton=1)
            order = sch["hex_order"].astype(np.uint32)
            stdin = struct.pack("<I", order.size) + order.tobytes()
            extra = {"order": order, "colour_hex_begin": sch["colour_hex_begin"]}
            if args[0] == "Qrings":
                rs = q.ring_schedule(morton=1)
                vorder = rs["vert_order"].astype(np.uint32)
                stdin += struct.pack("<I", vorder.size) + vorder.tobytes()
                extra.update(vorder=vorder, colour_vert_begin=rs["colour_vert_begin"])
        if args[0] in ("qordered", "qdamped", "qrings"):
            import oracle  # noqa: E402
            W, H, D, sx, sy, sz, pattern, wonk, dens = args[1:10]
            nodes, idx = oracle.gen_tet_block(W, H, D, (sx, sy, sz), pattern, wonk)
            q = oracle.Quadratic(nodes, idx, dens)
            sch = q.schedule(morton=1)
            order = sch["tet_order"].astype(np.uint32)
            stdin = struct.pack("<I", order.size) + order.tobytes()
            extra = {"order": order, "colour_tet_begin": sch["colour_tet_begin"]}
            if args[0] == "qrings":
                rs = q.ring_schedule(morton=1)
                vorder = rs["vert_order"].astype(np.uint32)
                stdin += struct.pack("<I", vorder.size) + vorder.tobytes()
                extra.update(vorder=vorder, colour_vert_begin=rs["colour_vert_begin"])
        if args[0] == "mixed":
            import oracle  # noqa: E402
            nodes, idx = mixed_mesh(args)
            tets, hexes, _ = oracle.parse_mixed(idx)
            ts = oracle.tet_element_schedule(nodes, tets, morton=1)
            hs = oracle.hex_schedule(nodes, hexes, morton=1)
            torder, horder = ts["tet_order"].astype(np.uint32), hs["hex_order"].astype(np.uint32)
            argv = [REFGEN, "mixed"] + [str(a) for a in args[10:]]
            stdin = (struct.pack("<I", nodes.size) + nodes.astype(np.float32).tobytes() + struct.pack("<I", idx.size) +
                     idx.astype(np.uint32).tobytes() + struct.pack("<I", torder.size) + torder.tobytes() +
                     struct.pack("<I", horder.size) + horder.tobytes())
            extra = {"torder": torder, "colour_tet_begin": ts["colour_tet_begin"], "horder": horder,
                     "colour_hex_begin": hs["colour_hex_begin"]}
        if args[0] == "qmixed":
            import oracle  # noqa: E402
            nodes, idx = mixed_mesh(args)
            sch = oracle.QuadraticMixed(nodes, idx, args[10]).schedules(morton=1)
            torder, horder = sch["t10_order"].astype(np.uint32), sch["h27_order"].astype(np.uint32)
            argv = [REFGEN, "qmixed"] + [str(a) for a in args[10:]]
            stdin = (struct.pack("<I", nodes.size) + nodes.astype(np.float32).tobytes() + struct.pack("<I", idx.size) +
                     idx.astype(np.uint32).tobytes() + struct.pack("<I", torder.size) + torder.tobytes() +
                     struct.pack("<I", horder.size) + horder.tobytes())
            extra = {"torder": torder, "colour_t10_begin": sch["colour_t10_begin"], "horder": horder,
                     "colour_h27_begin": sch["colour_h27_begin"]}
        if args[0] in ("ordered", "damped", "rings", "locked"):
            import oracle  # noqa: E402
            W, H, D, sx, sy, sz, wonk = args[1:8]
            nodes, idx = oracle.gen_tet_block(W, H, D, (sx, sy, sz), 0, wonk)
            tets, _ = oracle.parse_tets(idx)
            mode = 1 if name.endswith("_star") else 0
            sch = oracle.schedule(nodes, tets, mode=mode, morton=1)
            order = sch["tet_order"].astype(np.uint32)
            stdin = struct.pack("<I", order.size) + order.tobytes()
            extra = {"order": order, "colour_tet_begin": sch["colour_tet_begin"]}
            manifest_mode = mode
            if args[0] == "rings":
                rs = oracle.ring_schedule(nodes, tets, morton=1)
                vorder = rs["vert_order"].astype(np.uint32)
                stdin += struct.pack("<I", vorder.size) + vorder.tobytes()
                extra.update(vorder=vorder, colour_vert_begin=rs["colour_vert_begin"])
        r = subprocess.run(argv, input=stdin, stdout=subprocess.PIPE, check=True)
        arrays = parse(r.stdout)
        arrays.update(extra)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
        manifest[name] = {"args": args}
        if args[0] in ("ordered", "damped", "rings", "locked"):
            manifest[name]["schedule_mode"] = manifest_mode
        print(f"{name}: " + ", ".join(f"{k}{list(v.shape)}" for k, v in arrays.items()))
    manifest = {n: manifest[n] for n, _ in CASES if n in manifest}
    with open(mpath, "w") as f:
        json.dump(manifest, f, indent=1)


if __name__ == "__main__":
    main()
