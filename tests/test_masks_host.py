"""The interior fill and pivot masks compiled into the masked band solves
(vmask_*, vmask6_*, gmask_* in csrc/owt_device.cuh) are the ones the
derivation program (csrc/masks/derive_masks.cpp) finds from the production
band templates of the reference's eighth-order operators and of the
sixth-order option: built with g++ and run here, its output must equal the
compiled constants."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "open-3d-wallturbulence_gb300", "csrc")
OUT = os.path.join(ROOT, "oracle", "_build")


def _derive():
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "derive_masks")
    subprocess.run(["g++", "-std=c++17", "-O2", os.path.join(CSRC, "masks", "derive_masks.cpp"),
                    os.path.join(CSRC, "setup_host.cpp"), "-o", exe], check=True)
    return subprocess.run([exe], check=True, capture_output=True, text=True, timeout=300).stdout


def _order_block(text, order):
    blk = text.split(f"order {order}")[1].split("order ")[0]
    v = {k: [int(x, 16) for x in re.findall(r"0x[0-9a-f]+", re.search(rf"v {k}:([^\n]*)", blk).group(1))]
         for k in ("L", "U", "P")}
    g = re.search(r"g L:\s*(0x[0-9a-f]+) (0x[0-9a-f]+)\s+U:\s*(0x[0-9a-f]+) (0x[0-9a-f]+)", blk).groups()
    return v, [int(x, 16) for x in g]


def _compiled():
    src = open(os.path.join(CSRC, "owt_device.cuh")).read()

    def masks(name):
        body = re.search(rf"constexpr unsigned long long {name}\(int ty\) \{{(.*?)\}}", src, re.S).group(1)
        return body

    def eval_mask(body, ty):
        # the bodies are chains "ty == a ? X : ty == b ? Y : ... : Z"
        expr = body.replace("return", "").replace(";", "").replace("ull", "").strip()
        expr = re.sub(r"ty == (\d+) \? ", r"(\1 == TY) and ", expr)
        parts = re.split(r" : ", expr)
        for p in parts[:-1]:
            cond, val = p.split(" and ")
            if eval(cond.replace("TY", str(ty))):
                return int(val, 16)
        return int(parts[-1], 16)
    v = {k: [eval_mask(masks(f"vmask_{k.lower()}"), ty) for ty in range(4)] for k in ("L", "U", "P")}
    v6 = {k: [eval_mask(masks(f"vmask6_{k.lower()}"), ty) for ty in range(4)] for k in ("L", "U", "P")}
    g = [eval_mask(masks("gmask_l"), 0), eval_mask(masks("gmask_l"), 1),
         eval_mask(masks("gmask_u"), 0), eval_mask(masks("gmask_u"), 1)]
    return v, v6, g


def test_compiled_masks_are_the_derived_ones():
    try:
        text = _derive()
    except (OSError, subprocess.CalledProcessError) as e:  # no g++
        pytest.skip(f"cannot build the derivation program: {e}")
    want_v, want_v6, want_g = _compiled()
    got_v, got_g = _order_block(text, 8)
    assert got_v == want_v
    assert got_g == want_g
    got_v6, got_g6 = _order_block(text, 6)  # the sixth-order option: its own v masks, the same g masks
    assert got_v6 == want_v6
    assert got_g6 == want_g
