"""Source rules of the CUDA code that a compiler does not enforce.

A full-mask warp intrinsic (__shfl_*_sync, __ballot_sync, __any_sync,
__all_sync, __reduce_*_sync, __match_*_sync) must be executed by every lane
the mask names.  Written as one operand of a conditional expression
(`c ? __shfl_sync(...) : x`) it runs only on the lanes that pick that operand,
which is undefined behaviour and on the GPU can end the kernel with an
illegal-instruction fault.  The same holds for the right operand of && and ||.
"""

import pathlib
import re

CSRC = pathlib.Path(__file__).resolve().parents[1] / "bachelor-thesis_gb300" / "csrc"
WARP = r"__(?:shfl(?:_up|_down|_xor)?_sync|ballot_sync|any_sync|all_sync|reduce_\w+_sync|match_\w+_sync)\s*\("
BAD = re.compile(r"(?:\?|:(?!:)|&&|\|\|)\s*" + WARP)


def _code_lines(path):
    for n, line in enumerate(path.read_text().splitlines(), 1):
        code = line.split("//", 1)[0]
        if code.strip():
            yield n, code


def test_no_warp_intrinsic_in_a_conditional_operand():
    files = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cuh"))
    assert files
    bad = [f"{p.name}:{n}: {code.strip()}" for p in files for n, code in _code_lines(p) if BAD.search(code)]
    assert not bad, "warp intrinsic in a conditional operand:\n" + "\n".join(bad)


def test_rule_catches_the_pattern():
    assert BAD.search("const uint32_t e0 = lane == 31 ? __shfl_sync(kFull, s1, 0) : n0;")
    assert BAD.search("bool x = ok && __any_sync(kFull, v);")
    assert not BAD.search("const uint32_t s32 = __shfl_sync(kFull, s1, 0);")
    assert not BAD.search("case 1: x = 2;")
