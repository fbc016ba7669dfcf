"""GPU: uneven fields of every formula in one call (fractal_gb300_render_fields_device).

The batch workload mixes Mandelbrot, Julia, burning-ship and tricorn fields
of four sizes, zooms 1e10-1e100 and caps 1e4-1e6, with derivative planes.
Here the same seeded construction runs at an eighth of the sizes and caps up
to 1e5 so the test stays short.  Checks:

* form 0 (plain FP64) equals the per-field reference-ABI renders bit for bit,
  derivative planes included (the per-field renders' own parity with the
  reference is tested in test_gpu_parity.py);
* form 1 (the Mandelbrot fields in one persistent FP32 queue, the other
  formulas' in FP64 beside it) stays within 1e-4 of form 0's Mandelbrot
  counts (plus two pixels of slack) and equals form 0 elsewhere; its
  derivative planes are within a few parts per thousand where counts agree;
* the opt-in FP32 form of the other formulas (one queue for all four)
  renders without NaN and leaves the Mandelbrot fields unchanged;
* both against the reference's own deep fixtures of the other formulas
  (1e30-1e100, caps 1e5-1e6): form 1 exactly, the FP32 opt-in within a few
  pixels for tricorn (its Julia and burning-ship views drift, which a direct
  mpmath iteration attributes to FP32).
"""

from __future__ import annotations

import numpy as np
import pytest

from .conftest import golden_arrays
from .golden import cases as case_defs

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

MISMATCH_BUDGET = 1e-4
SMALL_SIZES = tuple((w // 8, h // 8) for w, h in case_defs.BATCH_SIZES)


def _field_set(package, product, mix):
    specs = [package.fields.FieldSpec(m["formula"], m["re"], m["im"], m["log10_zoom"], m["width"], m["height"],
                                      m["max_iter"], tuple(m["julia"])) for m in mix]
    return package.fields.FieldSet(product, specs)


def _buffers(mix):
    out = []
    for m in mix:
        n = m["width"] * m["height"]
        out.append((torch.full((n,), -1.0, dtype=torch.float32, device="cuda"),
                    torch.zeros((n,), dtype=torch.int32, device="cuda"),
                    torch.zeros((n,), dtype=torch.float64, device="cuda"),
                    torch.zeros((n,), dtype=torch.float64, device="cuda")))
    return out


def _targets(bufs):
    return [tuple(t.data_ptr() for t in b) for b in bufs]


def test_mixed_batch_in_one_call(package, product):
    mix = case_defs.batch_mix(seed=77, count=64, sizes=SMALL_SIZES, log_cap=(4.0, 5.0))
    assert {m["formula"] for m in mix} == {"mandelbrot", "julia", "burning-ship", "tricorn"}
    assert {(m["width"], m["height"]) for m in mix} == set(SMALL_SIZES)
    native = package.native
    fields = _field_set(package, product, mix)
    try:
        plain = _buffers(mix)
        fields.render_device(_targets(plain), form=0)
        chosen = _buffers(mix)
        fields.render_device(_targets(chosen), form=1, graph=True)
        fp32_all = _buffers(mix)
        fields.render_device(_targets(fp32_all), form=1, graph=True, fp32_alternates=True)
        torch.cuda.synchronize()
        # Form 0 against the per-field reference ABI with planes (host
        # buffers): fields, counts and derivative planes bit for bit.
        for i, m in enumerate(mix):
            zoom = fields.zooms[i]
            if m["log10_zoom"] < 12.0:
                want, planes = native.render_fractal(product, m["width"], m["height"], zoom, m["re"], m["im"],
                                                     m["max_iter"], 256, False, formula=m["formula"],
                                                     julia=tuple(float(v) for v in m["julia"]), planes=True)
            else:
                want, planes = native.render_reference(product, fields.handles[i], m["width"], m["height"], zoom,
                                                       m["max_iter"], planes=True)
            counts = native.iteration_counts(want, planes["orbit_iteration"], m["max_iter"])
            if m["formula"] == "julia" and m["log10_zoom"] >= 12.0:
                # The deep Julia orbit_iteration is the escape index itself.
                escaped = (counts > 0) & (counts < m["max_iter"])
                counts[escaped] -= 1
            f, c, dx, dy = (t.cpu().numpy() for t in plain[i])
            np.testing.assert_array_equal(f.view(np.uint32), want.view(np.uint32), err_msg=m["name"])
            np.testing.assert_array_equal(c.view(np.uint32), counts, err_msg=m["name"])
            np.testing.assert_array_equal(dx, planes["de_x"], err_msg=m["name"])
            np.testing.assert_array_equal(dy, planes["de_y"], err_msg=m["name"])
        # Form 1 against form 0, per formula.
        per_formula = {}
        per_field = []
        de_errors = []
        for m, p, q in zip(mix, plain, chosen):
            pc, qc = p[1].cpu().numpy(), q[1].cpu().numpy()
            differ, total = per_formula.get(m["formula"], (0, 0))
            n = int(np.count_nonzero(pc != qc))
            per_field.append((m["name"], round(m["log10_zoom"], 1), n))
            per_formula[m["formula"]] = (differ + n, total + pc.size)
            assert not np.isnan(q[0].cpu().numpy()).any(), m["name"]
            same = (pc == qc) & (pc < m["max_iter"])
            pd = np.hypot(p[2].cpu().numpy(), p[3].cpu().numpy())[same]
            qd = np.hypot(q[2].cpu().numpy(), q[3].cpu().numpy())[same]
            ok = pd > 0
            de_errors.append(np.abs(qd[ok] - pd[ok]) / pd[ok])
        worst = sorted(per_field, key=lambda t: -t[2])[:6]
        for formula, (differ, total) in per_formula.items():
            budget = MISMATCH_BUDGET * total + 2 if formula == "mandelbrot" else 0
            assert differ <= budget, (formula, differ, total, worst)
        for m, q, a in zip(mix, chosen, fp32_all):
            assert not np.isnan(a[0].cpu().numpy()).any(), m["name"]
            if m["formula"] == "mandelbrot":
                np.testing.assert_array_equal(a[1].cpu().numpy(), q[1].cpu().numpy(), err_msg=m["name"])
        de_errors = np.concatenate(de_errors)
        assert np.median(de_errors) <= 1e-3, np.median(de_errors)
        assert np.quantile(de_errors, 0.99) <= 5e-2, np.quantile(de_errors, 0.99)
    finally:
        fields.close()


@pytest.mark.parametrize("fp32", [False, True])
@pytest.mark.parametrize("case", case_defs.deep_alternate_cases(), ids=lambda c: c["name"])
def test_floatexp_alternates_against_deep_fixtures(package, product, case, fp32):
    """Form 1 of Julia, burning ship and tricorn at 1e30-1e100 (caps 1e5-1e6)
    against the reference's fixtures: exact by default (FP64), no NaN and,
    for tricorn, within a few pixels of 2304 with the FP32 opt-in."""
    stored = golden_arrays(case["name"])
    mix = [dict(name=case["name"], formula=case["formula"], re=case["centre"]["re"], im=case["centre"]["im"],
                julia=case.get("julia", ("0", "0")), log10_zoom=case["log10_zoom"], width=case["width"],
                height=case["height"], max_iter=case["max_iter"])]
    fields = _field_set(package, product, mix)
    try:
        bufs = _buffers(mix)
        fields.render_device(_targets(bufs), form=1, fp32_alternates=fp32)
        torch.cuda.synchronize()
    finally:
        fields.close()
    got = bufs[0][1].cpu().numpy().view(np.uint32)
    want = stored["counts"].copy()
    if case["formula"] == "julia":
        escaped = (want > 0) & (want < case["max_iter"])
        want[escaped] -= 1
    assert not np.isnan(bufs[0][0].cpu().numpy()).any()
    differ = got != want
    if not fp32:
        np.testing.assert_array_equal(got, want)
    elif case["formula"] == "tricorn":
        assert np.count_nonzero(differ) <= 1e-3 * want.size + 2, (
            np.count_nonzero(differ), got[differ][:8].tolist(), want[differ][:8].tolist())
