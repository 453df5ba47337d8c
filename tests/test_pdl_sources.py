"""Programmatic dependent launches (pdl_launch, or the
cudaLaunchAttributeProgrammaticStreamSerialization attribute) let a kernel be
scheduled while the kernel before it on the stream still runs.  Such a
kernel is only correct if it waits (griddepcontrol.wait) before it touches
any data.  This source check finds every kernel the library launches that
way and asserts that its body opens with the wait."""
import glob
import os
import re

import pytest

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "peeeeeeeeeeeeeeeeeeec_gb300",
                    "csrc")
WAIT = re.compile(r"^\s*(pdl_wait\(\);|asm volatile\(\"griddepcontrol\.wait;\"[^;]*;)")


def sources():
    out = {}
    for p in sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cuh"))):
        with open(p) as f:
            out[os.path.basename(p)] = f.read()
    return out


def pdl_kernels(src):
    names = set()
    for text in src.values():
        for m in re.finditer(r"pdl_launch\(\s*([A-Za-z_:][A-Za-z_0-9:]*)", text):
            names.add(m.group(1).split("::")[-1])
        # launches that set the attribute themselves name the kernel in their cudaLaunchKernelEx call
        for m in re.finditer(r"cudaLaunchAttributeProgrammaticStreamSerialization", text):
            tail = text[m.end():m.end() + 800]
            k = re.search(r"cudaLaunchKernelEx\(&cfg,\s*([A-Za-z_][A-Za-z_0-9]*)", tail)
            if k:
                names.add(k.group(1))
    names.discard("kernel")  # the helper's own parameter (and its declaration)
    names.discard("void")
    return names


def kernel_body_opening(src, name):
    for text in src.values():
        for m in re.finditer(r"__global__\s+void\s+(?:__launch_bounds__\([^)]*\)\s+)?\s*" + re.escape(name) + r"\(",
                             text):
            brace = text.index("{", m.end())
            return text[brace + 1:brace + 400].lstrip("\n")
    return None


def test_every_programmatic_dependent_waits_first():
    src = sources()
    names = pdl_kernels(src)
    assert {"k_panel_cl", "k_laswp", "k_trsm", "k_split_a", "k_split_b", "k_tc_gemm_cplx_persistent",
            "k_minv_apply", "k_transient_rhs"} <= names, names
    for name in sorted(names):
        body = kernel_body_opening(src, name)
        assert body is not None, "kernel %s not found" % name
        first = [line for line in body.splitlines() if line.strip() and not line.strip().startswith("//")][0]
        assert WAIT.match(first), "%s does not open with the dependency wait: %r" % (name, first)


@pytest.mark.parametrize("name", ["k_trsv_wave"])
def test_ticket_ordered_solve_is_an_ordinary_launch(name):
    """The triangular solve takes its blocks in ticket order and needs no
    co-residency: it is not a cooperative launch."""
    src = sources()
    for text in src.values():
        assert not re.search(r"cudaLaunchCooperativeKernel\([^;]*" + name, text), name
