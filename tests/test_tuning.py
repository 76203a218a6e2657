"""CPU checks of the pass-line tuning: the autotuner's class naming, and the
committed tuning header defines a well-formed line for every key/value class
in both size classes (the build takes the header over the defaults)."""
import os
import re
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "x86-simd-sort_gb300")
sys.path.insert(0, PKG)

import autotune  # noqa: E402


def test_class_names_map_to_macros():
    assert autotune._base("K32") == ("K32", "XSS_CFG_K32", False)
    assert autotune._base("K64V64_MID") == ("K64V64", "XSS_CFGM_K64V64", True)
    for cls in autotune.CANDIDATES:
        base, _, _ = autotune._base(cls)
        assert base in autotune.CLASSES, cls


def test_candidate_lines_are_well_formed():
    for cls, lines in autotune.CANDIDATES.items():
        for line in lines:
            f = [int(x) for x in line.split(",")]
            assert len(f) == 7, (cls, line)
            block, items, minb, lb, rank, persist, dpt = f
            assert block % 32 == 0 and 256 <= block <= 1024
            assert items >= 1 and minb >= 1 and lb in (8, 16, 32)
            assert rank in (0, 1, 2) and persist in (0, 1, 2, 3) and dpt in (0, 1, 2, 4, 12, 14)


def test_committed_header_covers_every_class():
    text = open(os.path.join(PKG, "csrc", "xss_tuning.h")).read()
    lines = dict(re.findall(r"#define (XSS_CFGM?_\w+) ([0-9, ]+)\n", text))
    for cls in autotune.CLASSES:
        for macro in ("XSS_CFG_" + cls, "XSS_CFGM_" + cls):
            assert macro in lines, macro
            f = [int(x) for x in lines[macro].split(",")]
            assert len(f) == 7 and f[0] % 32 == 0 and f[4] in (0, 1, 2)


def test_a_candidate_line_builds_into_its_own_library():
    """The tuner's variant build (one pre-included line, the radix unit
    recompiled, linked with the shared objects) works without a GPU."""
    common = autotune.build_common()
    so = autotune.build_variant("K32", "320,20,3,8,2,1,0", common)
    assert os.path.exists(so) and os.path.getsize(so) > 0
