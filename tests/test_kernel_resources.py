"""Register budgets of the step's kernels, read from ptxas's resource report of
the in-tree build (no GPU needed).

The kernels are sized for residency: the render forward and one-pass backward at
48 registers (10 blocks of 128 threads per SM); MacCormack forward 1 at 32
(8 blocks of 256) and backward 2 at 48 (5 blocks of 256), the same for 16-bit
storage as for f32.  One register more costs a resident block per SM, so a
change that crosses a budget fails here rather than only in a timing run.
"""
import os
import re

import pytest

import __graft_entry__


@pytest.fixture(scope="module")
def reports():
    __graft_entry__.load_package()
    from ngt_gb300 import _build
    # the step's advection kernels, the render kernels of float storage, and the
    # raymarch host unit's quad build and fold
    srcs = [os.path.join(_build.CSRC, n) for n in ("advect.cu", "raymarch_f32.cu", "raymarch.cu")]
    _build.build_library()  # rebuilds (and rewrites the reports) when a source is newer than the library
    if not all(os.path.exists(_build.resource_report(s)) for s in srcs):
        _build.build_library(force=True)
    out = {}
    for s in srcs:
        out.update({(os.path.basename(s), k): v for k, v in parse(open(_build.resource_report(s)).read()).items()})
    return out


def parse(text):
    """{mangled kernel name: (registers, spill store bytes, spill load bytes)}"""
    res, cur, spill = {}, None, (0, 0)
    for line in text.splitlines():
        m = re.search(r"Compiling entry function '([^']+)'", line)
        if m:
            cur, spill = m.group(1), (0, 0)
            continue
        m = re.search(r"(\d+) bytes spill stores, (\d+) bytes spill loads", line)
        if m and cur:
            spill = (int(m.group(1)), int(m.group(2)))
        m = re.search(r"Used (\d+) registers", line)
        if m and cur:
            res[cur] = (int(m.group(1)),) + spill
            cur = None
    return res


def find(reports, *parts, source=None):
    hits = [v for (src, k), v in reports.items() if all(p in k for p in parts) and source in (None, src)]
    assert len(hits) == 1, (parts, len(hits))
    return hits[0]


# storage type of the density, and of the lookup's faces (the same type: "IfE" or,
# for 16-bit types, the substitution "IS2_E")
STORAGE = {"f32": ("f", "IfE"), "bf16": ("13__nv_bfloat16", "IS2_E"), "f16": ("6__half", "IS2_E")}


@pytest.mark.parametrize("storage", sorted(STORAGE))
def test_maccormack_register_budgets(reports, storage):
    t, faces = STORAGE[storage]
    regs, st, ld = find(reports, "k_mc_fwd1ILi1E" + t + "NS0_14CenteredLookup" + faces)
    assert regs <= 32 and st == ld == 0
    regs, st, ld = find(reports, "k_mc_bwd2ILi1E" + t + "NS0_12StoredLookup")
    assert regs <= 48 and st == ld == 0


# the render kernels come in two instances: rays read from a prepared table (Li1E)
# and rays set up in the kernel (Li2E)
@pytest.mark.parametrize("kernel", ["k_raymarch_fwdILi1ELi2EffLi1EE", "k_raymarch_fwdILi1ELi2EffLi2EE",
                                    "k_raymarch_bwd_blILi1ELi2EffLi2EE"])
def test_render_register_budgets(reports, kernel):
    regs, st, ld = find(reports, kernel)
    assert regs <= 48 and st == ld == 0


def test_render_backward_table_instance(reports):
    """The one-pass backward that reads prepared rays stays at 48 registers; the
    few bytes it keeps in local memory are saved around its call of the
    checkpointed adjoint (taken only when the extinction-sign check fails):
    without that call it has none."""
    regs, st, ld = find(reports, "k_raymarch_bwd_blILi1ELi2EffLi1EE")
    assert regs <= 48 and st <= 32 and ld <= 32


def test_quad_kernels_do_not_spill(reports):
    for k in ("k_quad_foldEPK6float4", "k_quad_buildIfEE"):
        _, st, ld = find(reports, k, source="raymarch.cu")
        assert st == ld == 0
