"""Cases of the golden fixtures: reference-exact settings (pillbox sun, reflectivity 1, no slope
or specularity error), the only physics the reference implements."""
import numpy as np

from optixsoltracedemos_gb300 import scenes


def three_heliostats():
    return scenes.three_heliostats(reflectivity=1.0, slope_error=0.0), 2048, 0, 0, 0


def three_heliostats_seed7():
    return scenes.three_heliostats(reflectivity=1.0, slope_error=0.0), 1024, 7, 3, 5000


def parabolic_cylinder():
    sc = scenes.single_parabolic(sun_shape=scenes.SUN_PILLBOX, sun_sigma=4.65e-3, slope_error=0.0)
    return sc, 2048, 0, 0, 0


def toy_problem_parabolic():
    """The element list of the reference's data/stinput/toy_problem_parabolic.stinput (three
    parabolic 1 x 1.95 m heliostats, flat 2 x 2 receiver at z = 10, sun (0,0,100), 4.65 mrad
    pillbox), entered by hand from the file's element lines."""
    e = scenes.make_elements(4)
    e["origin"][:3] = [[-5.0, 0.0, 0.0], [0.0, 5.0, 0.0], [5.0, 0.0, 0.0]]
    e["aim_point"][:3] = [[17.360680, -0.0, 94.721360], [0.0, -17.360680, 94.721360], [-17.360680, -0.0, 94.721360]]
    e["zrot_deg"][:3] = [-88.757211, -0.0, 88.757211]
    e["width"][:3] = 1.0
    e["height"][:3] = 1.95
    e["curv_x"][:3] = 0.017068
    e["curv_y"][:3] = 0.037068
    e["surface"][:3] = scenes.SURFACE_PARABOLIC
    e["origin"][3] = [0.0, 0.0, 10.0]
    e["aim_point"][3] = [0.0, 5.0, 0.0]
    e["width"][3] = 2.0
    e["height"][3] = 2.0
    e["surface"][3] = scenes.SURFACE_FLAT
    sc = scenes.Scene("toy_problem_parabolic", e, np.array([0.0, 0.0, 100.0]), scenes.SUN_PILLBOX, 4.65e-3, 2048)
    return sc, 2048, 0, 0, 0


def small_field():
    sc = scenes.large_field(n_heliostats=60, slope_error=0.0, sun=scenes.sun_vector(30.0, 20.0))
    return sc, 2048, 1, 0, 0


CASES = {
    "three_heliostats": three_heliostats,
    "three_heliostats_seed7": three_heliostats_seed7,
    "parabolic_cylinder": parabolic_cylinder,
    "toy_problem_parabolic": toy_problem_parabolic,
    "small_field": small_field,
}
