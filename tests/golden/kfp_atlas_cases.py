"""Atlas KFP parity cases: fractal_atlas_colourise_kfp (separate tiles at
output scale) and fractal_atlas_colourise_kfp_planes (reprojected surface and
render planes, one plane-aware KFP pass).

Sources are stored parity fields and their render planes (``fixtures/*.npz``);
the separate-tile child is a crop of another field, the plane-atlas sources
are whole fields (centred cases store them relative to their own cap).
Options are the package's named KFP recipes with overrides; LUTs are the
reference's (``fixtures/kfp_luts.npz``).  ``run`` drives any library
exporting the renderer.h ABI.
"""

from __future__ import annotations

import os

import numpy as np

from .kfp_planes_cases import FIELDS, SIZES, texture
from .runner import _native

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = os.path.join(HERE, "fixtures")
KFP_ATLAS_FIXTURE = os.path.join(FIXTURES, "kfp_atlas.npz")


def _tiles(name, parent, child, origin, feather, recipe, marks=False, **overrides):
    """Separate tiles: `child` = (field, x0, y0, width, height) crop; `marks`
    stamps interior blocks (value = max_iter) into both tiles."""
    return dict(name=name, kind="tiles", parent=parent, child=child, origin=origin, feather=feather, recipe=recipe,
                marks=marks, overrides=overrides)


def _planes(name, parent, child, output, parent_zoom, fraction, child_zoom, recipe, centered=0,
            parent_set="orbit", child_set="orbit", texture_spec=None, **overrides):
    return dict(name=name, kind="planes", parent=parent, child=child, output=output, parent_zoom=parent_zoom,
                fraction=fraction, child_zoom=child_zoom, recipe=recipe, centered=centered, parent_set=parent_set,
                child_set=child_set, texture=texture_spec, overrides=overrides)


def kfp_atlas_cases() -> list[dict]:
    e100 = "e100_bias_64x36"
    nobla = "e100_nobla_64x36"
    deep = "deep_p80_e32_block32_64x36"
    cases = []
    for recipe in ("default", "seeded16", "method4", "multicolor", "differences7"):
        cases.append(_tiles(f"tiles_{recipe}_feather6", e100, (deep, 10, 5, 40, 24), (12, 6), 6, recipe,
                            marks=recipe == "seeded16"))
    cases += [
        _tiles("tiles_feather0", e100, (deep, 3, 2, 37, 23), (20, 9), 0, "seeded16", marks=True),
        _tiles("tiles_feather1", e100, (deep, 3, 2, 37, 23), (20, 9), 1, "default", marks=True),
        _tiles("tiles_feather_max", e100, (deep, 10, 8, 30, 20), (0, 0), 20, "default"),
        _tiles("tiles_corner", e100, (deep, 30, 10, 34, 26), (30, 10), 4, "method4", marks=True),
        _tiles("tiles_full_child", e100, (deep, 0, 0, 64, 36), (0, 0), 8, "seeded16"),
        _tiles("tiles_no_child", e100, None, (0, 0), 0, "default"),
        _tiles("tiles_slopes_odd", e100, (deep, 5, 5, 27, 17), (9, 11), 5, "default", slope_power=40.0),
    ]
    for recipe in ("default", "seeded16", "differences7", "method4", "multicolor"):
        cases.append(_planes(f"planes_atlas_{recipe}", nobla, deep, (96, 54), 1.6, 0.5, 1.3, recipe))
    cases += [
        _planes("planes_atlas_centred", nobla, deep, (96, 54), 1.25, 0.6, 1.1, "default", centered=1,
                field_bias=200_000.0),
        _planes("planes_atlas_full_child", nobla, deep, (80, 45), 1.5, 1.0, 1.2, "seeded16"),
        _planes("planes_atlas_no_child", nobla, None, (80, 45), 1.7, 0.0, 1.0, "differences7"),
        _planes("planes_atlas_small_child", e100, deep, (96, 54), 2.0, 0.25, 1.0, "default"),
        _planes("planes_atlas_iteration_hidden", nobla, deep, (96, 54), 1.4, 0.5, 1.5, "seeded16",
                parent_set="iteration", child_set="iteration", show_glitches=0),
        _planes("planes_atlas_mixed_sets", nobla, deep, (96, 54), 1.4, 0.5, 1.5, "differences7",
                parent_set="orbit+bailout", child_set="de+phase"),
        _planes("planes_atlas_texture", nobla, deep, (96, 54), 1.3, 0.5, 1.2, "default",
                texture_spec=(60, 40, 3), texture_enabled=1, texture_merge=0.5, texture_power=16.0,
                texture_ratio=70.0),
        _planes("planes_atlas_phase", nobla, "odd_37x23", (96, 54), 1.3, 0.4, 1.0, "multicolor",
                phase_color_strength=45.0),
    ]
    return cases


def _stored(name):
    return np.load(os.path.join(FIXTURES, name + ".npz"))


def plane_set(name: str, kind: str) -> dict:
    """Render planes of stored field `name`: "orbit" (orbit_iteration, phase,
    de_x, de_y, test1, test2), "orbit+bailout", "iteration" (iteration +
    transition with 5 % hidden-glitch markers + phase), "de+phase"."""
    stored = _stored(name)
    max_iter, bias = FIELDS[name]
    if kind.startswith("orbit"):
        planes = {key: stored[key] for key in ("orbit_iteration", "phase", "de_x", "de_y", "test1", "test2")}
        if kind == "orbit+bailout":
            rng = np.random.default_rng(17)
            planes["bailout"] = rng.uniform(2.0, 1.0e6, size=planes["phase"].size)
        return planes
    if kind == "iteration":
        rng = np.random.default_rng(18)
        field = np.nan_to_num(stored["field"].astype(np.float64) + bias, nan=0.0)
        transition = 1.0 - (field - np.floor(field))
        transition[rng.uniform(size=field.size) < 0.05] = -1.0
        return {"iteration": np.floor(field).astype(np.int64), "transition": transition, "phase": stored["phase"]}
    if kind == "de+phase":
        return {"de_x": stored["de_x"], "de_y": stored["de_y"], "phase": stored["phase"]}
    raise ValueError(kind)


def _options(case):
    from .make_golden import _package_kfp

    kfp = _package_kfp()
    bias = case["overrides"].get("field_bias", FIELDS[case["parent"]][1] if case["kind"] == "tiles" else 0.0)
    options = kfp.options(kfp.recipe(case["recipe"]), field_bias=bias)
    for key, value in case["overrides"].items():
        setattr(options, key, value)
    with np.load(os.path.join(FIXTURES, "kfp_luts.npz")) as luts:
        lut = luts[case["recipe"]]
    return options, lut


def run(library, case: dict) -> np.ndarray:
    native = _native()
    options, lut = _options(case)
    if case["kind"] == "tiles":
        parent = _stored(case["parent"])["field"]
        width, height = SIZES[case["parent"]]
        max_iter = FIELDS[case["parent"]][0]
        child = child_shape = None
        if case["marks"]:
            parent = parent.copy().reshape(height, width)
            parent[14:20, 24:34] = np.float32(max_iter)
            parent = parent.ravel()
        if case["child"] is not None:
            name, x0, y0, cw, ch = case["child"]
            sw, _ = SIZES[name]
            whole = _stored(name)["field"].reshape(-1, sw)
            child = np.ascontiguousarray(whole[y0:y0 + ch, x0:x0 + cw])
            if case["marks"]:
                child[2:9, 3:12] = np.float32(max_iter)
                child[ch - 4:ch, cw - 6:cw] = np.float32(max_iter)
            child = child.ravel()
            child_shape = (cw, ch)
        return native.atlas_colourise_kfp(library, parent, (width, height), child, child_shape, case["origin"],
                                          case["feather"], max_iter, options, lut)
    parent_name, child_name = case["parent"], case["child"]
    parent_max, _ = FIELDS[parent_name]
    parent = _stored(parent_name)["field"]
    if case["centered"]:
        parent = (parent.astype(np.float64) - parent_max).astype(np.float32)
    parent_planes = plane_set(parent_name, case["parent_set"])
    child = child_planes = None
    child_shape, child_max = (0, 0), 0
    if child_name is not None:
        child_max, _ = FIELDS[child_name]
        child = _stored(child_name)["field"]
        if case["centered"]:
            child = (child.astype(np.float64) - child_max).astype(np.float32)
        child_planes = plane_set(child_name, case["child_set"])
        child_shape = SIZES[child_name]
    if case["texture"] is not None:
        parent_planes["texture"] = texture(case["texture"])
    return native.atlas_colourise_kfp_planes(
        library, parent, SIZES[parent_name], parent_max, parent_planes, child, child_shape, child_max, child_planes,
        case["output"], case["parent_zoom"], case["fraction"], case["child_zoom"], parent_max, case["centered"],
        options, lut)
