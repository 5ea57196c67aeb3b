"""Helpers shared by the parity tests: build one workload on the GPU library
and on the CPU oracle with identical calls, render, and compare.

Parity bar (stated by the benchmark spec for this path): coverage and depth bit-exact;
colour within 1 LSB per RGBA8 channel or 1e-5 relative for float targets.
The implementations are designed to agree exactly, and the tests also report
how many colour values differ at all.
"""
import numpy as np

RGBA8_TOL = 1          # LSB per channel
FLOAT_RTOL = 1e-5      # relative, float colour targets


def render_both(builder, gpu_ctx, oracle_ctx, frames=1, **kw):
    sg = builder(gpu_ctx, **kw)
    so = builder(oracle_ctx, **kw)
    for _ in range(frames):
        sg.render()
        so.render()
    gpu_ctx.finish()
    return sg, so


def compare_scenes(sg, so, label=""):
    """Depth bit-exact, then every colour attachment; returns the number of
    colour values of attachment 0 that differ at all."""
    dg, do = sg.read_depth(), so.read_depth()
    # depth: bit-exact (covers coverage and depth-test outcomes). A NaN depth
    # (written by a zero-area triangle when the depth test is off) matches any
    # NaN: each ISA produces its own NaN payload (x86 sets the sign bit).
    bits = {2: np.uint16, 4: np.uint32, 8: np.uint64}[dg.dtype.itemsize]
    bad = (dg.view(bits) != do.view(bits)) & ~(np.isnan(dg) & np.isnan(do))
    assert not bad.any(), f"{label}: {int(bad.sum())} depth texels differ, first at {np.argwhere(bad)[:3].tolist()}"
    for k in range(1, len(sg.attachments)):
        compare_colors(sg.read_color(k), so.read_color(k), f"{label} attachment {k}")
    return compare_colors(sg.read_color(), so.read_color(), label)


def compare_colors(cg, co, label=""):
    """8-bit channels within 1 LSB, wider integer channels exact, float
    channels within 1e-5 relative (NaN matches NaN)."""
    assert cg.dtype == co.dtype and cg.shape == co.shape, f"{label}: {cg.dtype}{cg.shape} vs {co.dtype}{co.shape}"
    if cg.dtype == np.uint8:
        diff = np.abs(cg.astype(np.int16) - co.astype(np.int16))
        assert diff.max(initial=0) <= RGBA8_TOL, f"{label}: colour differs by {diff.max()} LSB at {np.argwhere(diff > RGBA8_TOL)[:3].tolist()}"
        return int((diff > 0).sum())
    if cg.dtype.kind == "u":
        bad = cg != co
        assert not bad.any(), f"{label}: {int(bad.sum())} integer colour values differ, first at {np.argwhere(bad)[:3].tolist()}"
        return 0
    a, b = cg.astype(np.float64), co.astype(np.float64)
    scale = np.maximum(np.abs(b), 1e-30)
    rel = np.abs(a - b) / scale
    ok = (np.abs(a - b) <= FLOAT_RTOL * scale) | (a == b) | (np.isnan(a) & np.isnan(b))
    assert ok.all(), f"{label}: float colour rel err {np.nanmax(rel)}"
    bits = {2: np.uint16, 4: np.uint32, 8: np.uint64}[cg.dtype.itemsize]
    return int((cg.view(bits) != co.view(bits)).sum())
