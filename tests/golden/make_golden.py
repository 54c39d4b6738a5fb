"""Generate the known-answer fixtures under tests/golden/.

lcg.json: outputs of the reference's LCG<4> random generator
(common.h:55-102 in anari-visionaray) for fixed seeds, computed here by an
independent pure-Python restatement of its integer arithmetic (TEA-style
seed mixing, then state = 1664525*state + 1013904223, value = low 24 bits
/ 2^24). The oracle's C++ generator is checked against these values.

Run: python tests/golden/make_golden.py
"""
import json
import os

M = 0xFFFFFFFF


def lcg_init(v0, v1):
    s0 = 0
    for _ in range(4):
        s0 = (s0 + 0x9E3779B9) & M
        v0 = (v0 + ((((v1 << 4) & M) + 0xA341316C) & M ^ ((v1 + s0) & M) ^ (((v1 >> 5) + 0xC8013EA4) & M))) & M
        v1 = (v1 + ((((v0 << 4) & M) + 0xAD90777D) & M ^ ((v0 + s0) & M) ^ (((v0 >> 5) + 0x7E95761E) & M))) & M
    return v0


def lcg_sequence(v0, v1, n):
    st = lcg_init(v0, v1)
    out = []
    for _ in range(n):
        st = (1664525 * st + 1013904223) & M
        out.append((st & 0x00FFFFFF) / float(0x01000000))
    return out


if __name__ == "__main__":
    seeds = [(0, 0), (1, 0), (0, 1), (12345, 7), (1048575, 1023), (0xFFFFFFFF, 0xFFFFFFFF)]
    data = [{"seed": list(s), "values": lcg_sequence(s[0], s[1], 16)} for s in seeds]
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lcg.json")
    with open(path, "w") as f:
        json.dump(data, f, indent=1)
    print("wrote", path)
