"""ctypes mirror of the flam3 public structs (flam3.h:185-614, isaac.h:23-31).

The layout is byte-identical to the reference's (checked against offsets
printed from the real header, tests/golden/abi_offsets.txt), so the same
in-memory flam3_frame can be handed to the reference library, to the test
oracle and to libflam3gpu.
"""
import ctypes as C

NVARS = 99
RANDSIZ = 16

VARIATION_NAMES = [
    "linear", "sinusoidal", "spherical", "swirl", "horseshoe", "polar", "handkerchief", "heart",
    "disc", "spiral", "hyperbolic", "diamond", "ex", "julia", "bent", "waves", "fisheye", "popcorn",
    "exponential", "power", "cosine", "rings", "fan", "blob", "pdj", "fan2", "rings2", "eyefish",
    "bubble", "cylinder", "perspective", "noise", "julian", "juliascope", "blur", "gaussian_blur",
    "radial_blur", "pie", "ngon", "curl", "rectangles", "arch", "tangent", "square", "rays", "blade",
    "secant2", "twintrian", "cross", "disc2", "super_shape", "flower", "conic", "parabola", "bent2",
    "bipolar", "boarders", "butterfly", "cell", "cpow", "curve", "edisc", "elliptic", "escher", "foci",
    "lazysusan", "loonie", "pre_blur", "modulus", "oscilloscope", "polar2", "popcorn2", "scry",
    "separation", "split", "splits", "stripes", "wedge", "wedge_julia", "wedge_sph", "whorl", "waves2",
    "exp", "log", "sin", "cos", "tan", "sec", "csc", "cot", "sinh", "cosh", "tanh", "sech", "csch",
    "coth", "auger", "flux", "mobius",
]
VAR_INDEX = {n: i for i, n in enumerate(VARIATION_NAMES)}


class randctx(C.Structure):
    _fields_ = [
        ("randcnt", C.c_ulong),
        ("randrsl", C.c_ulong * RANDSIZ),
        ("randmem", C.c_ulong * RANDSIZ),
        ("randa", C.c_ulong),
        ("randb", C.c_ulong),
        ("randc", C.c_ulong),
    ]


class flam3_palette_entry(C.Structure):
    _fields_ = [("index", C.c_double), ("color", C.c_double * 4)]


class stat_struct(C.Structure):
    _fields_ = [("badvals", C.c_double), ("num_iters", C.c_long), ("render_seconds", C.c_int)]


# Variation parameters in declaration order (flam3.h:240-407), all double.
XFORM_PARAMS = (
    "blob_low blob_high blob_waves pdj_a pdj_b pdj_c pdj_d fan2_x fan2_y rings2_val "
    "perspective_angle perspective_dist julian_power julian_dist juliascope_power juliascope_dist "
    "radial_blur_angle pie_slices pie_rotation pie_thickness ngon_sides ngon_power ngon_circle "
    "ngon_corners curl_c1 curl_c2 rectangles_x rectangles_y amw_amp disc2_rot disc2_twist "
    "super_shape_rnd super_shape_m super_shape_n1 super_shape_n2 super_shape_n3 super_shape_holes "
    "flower_petals flower_holes conic_eccentricity conic_holes parabola_height parabola_width "
    "bent2_x bent2_y bipolar_shift cell_size cpow_r cpow_i cpow_power curve_xamp curve_yamp "
    "curve_xlength curve_ylength escher_beta lazysusan_spin lazysusan_space lazysusan_twist "
    "lazysusan_x lazysusan_y modulus_x modulus_y oscope_separation oscope_frequency "
    "oscope_amplitude oscope_damping popcorn2_x popcorn2_y popcorn2_c separation_x "
    "separation_xinside separation_y separation_yinside split_xsize split_ysize splits_x splits_y "
    "stripes_space stripes_warp wedge_angle wedge_hole wedge_count wedge_swirl wedge_julia_angle "
    "wedge_julia_count wedge_julia_power wedge_julia_dist wedge_sph_angle wedge_sph_count "
    "wedge_sph_hole wedge_sph_swirl whorl_inside whorl_outside waves2_freqx waves2_scalex "
    "waves2_freqy waves2_scaley auger_sym auger_weight auger_freq auger_scale flux_spread "
    "mobius_re_a mobius_im_a mobius_re_b mobius_im_b mobius_re_c mobius_im_c mobius_re_d mobius_im_d"
).split()

# Values derived by xform_precalc (flam3.h:409-441).
XFORM_DERIVED = (
    "persp_vsin persp_vfcos julian_rN julian_cn juliascope_rN juliascope_cn wedgeJulia_rN "
    "wedgeJulia_cn wedgeJulia_cf radialBlur_spinvar radialBlur_zoomvar waves_dx2 waves_dy2 "
    "disc2_sinadd disc2_cosadd disc2_timespi super_shape_pm_4 super_shape_pneg1_n1"
).split()


class flam3_xform(C.Structure):
    pass


flam3_xform._fields_ = (
    [
        ("var", C.c_double * NVARS),
        ("c", (C.c_double * 2) * 3),
        ("post", (C.c_double * 2) * 3),
        ("density", C.c_double),
        ("color", C.c_double),
        ("color_speed", C.c_double),
        ("animate", C.c_double),
        ("opacity", C.c_double),
        ("vis_adjusted", C.c_double),
        ("padding", C.c_int),
        ("wind", C.c_double * 2),
        ("precalc_angles_flag", C.c_int),
        ("precalc_atan_xy_flag", C.c_int),
        ("precalc_atan_yx_flag", C.c_int),
        ("has_preblur", C.c_double),
        ("has_post", C.c_int),
    ]
    + [(n, C.c_double) for n in XFORM_PARAMS]
    + [(n, C.c_double) for n in XFORM_DERIVED]
    + [
        ("num_active_vars", C.c_int),
        ("active_var_weights", C.c_double * NVARS),
        ("varFunc", C.c_int * NVARS),
        ("motion_freq", C.c_int),
        ("motion_func", C.c_int),
        ("motion", C.POINTER(flam3_xform)),
        ("num_motion", C.c_int),
    ]
)


class flam3_genome(C.Structure):
    _fields_ = [
        ("flame_name", C.c_char * 65),
        ("time", C.c_double),
        ("interpolation", C.c_int),
        ("interpolation_type", C.c_int),
        ("palette_interpolation", C.c_int),
        ("hsv_rgb_palette_blend", C.c_double),
        ("num_xforms", C.c_int),
        ("final_xform_index", C.c_int),
        ("final_xform_enable", C.c_int),
        ("xform", C.POINTER(flam3_xform)),
        ("chaos", C.POINTER(C.POINTER(C.c_double))),
        ("chaos_enable", C.c_int),
        ("genome_index", C.c_int),
        ("parent_fname", C.c_char * 30),
        ("symmetry", C.c_int),
        ("palette", flam3_palette_entry * 256),
        ("input_image", C.c_char_p),
        ("palette_index", C.c_int),
        ("brightness", C.c_double),
        ("contrast", C.c_double),
        ("gamma", C.c_double),
        ("highlight_power", C.c_double),
        ("width", C.c_int),
        ("height", C.c_int),
        ("spatial_oversample", C.c_int),
        ("center", C.c_double * 2),
        ("rot_center", C.c_double * 2),
        ("rotate", C.c_double),
        ("vibrancy", C.c_double),
        ("hue_rotation", C.c_double),
        ("background", C.c_double * 3),
        ("zoom", C.c_double),
        ("pixels_per_unit", C.c_double),
        ("spatial_filter_radius", C.c_double),
        ("spatial_filter_select", C.c_int),
        ("sample_density", C.c_double),
        ("nbatches", C.c_int),
        ("ntemporal_samples", C.c_int),
        ("estimator", C.c_double),
        ("estimator_curve", C.c_double),
        ("estimator_minimum", C.c_double),
        ("edits", C.c_void_p),
        ("gam_lin_thresh", C.c_double),
        ("palette_index0", C.c_int),
        ("hue_rotation0", C.c_double),
        ("palette_index1", C.c_int),
        ("hue_rotation1", C.c_double),
        ("palette_blend", C.c_double),
        ("temporal_filter_type", C.c_int),
        ("temporal_filter_width", C.c_double),
        ("temporal_filter_exp", C.c_double),
        ("palette_mode", C.c_int),
    ]


PROGRESS_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_double, C.c_int, C.c_double)


class flam3_frame(C.Structure):
    _fields_ = [
        ("pixel_aspect_ratio", C.c_double),
        ("genomes", C.POINTER(flam3_genome)),
        ("ngenomes", C.c_int),
        ("verbose", C.c_int),
        ("bits", C.c_int),
        ("bytes_per_channel", C.c_int),
        ("earlyclip", C.c_int),
        ("time", C.c_double),
        ("progress", PROGRESS_FN),
        ("progress_parameter", C.c_void_p),
        ("rc", randctx),
        ("nthreads", C.c_int),
        ("sub_batch_size", C.c_int),
    ]


def layout_report():
    """Lines in the format of oracle/abi_offsets.c for the checked fields."""
    out = []
    for t in (randctx, flam3_palette_entry, stat_struct, flam3_xform, flam3_genome, flam3_frame):
        out.append(f"sizeof {t.__name__} {C.sizeof(t)}")
    return out


def offset_of(struct, field):
    return getattr(struct, field).offset
