"""Extract the LG exchangeability matrix and frequencies into ``lg.dat``.

LG (Le & Gascuel 2008) is a published empirical protein model. IQ-TREE 2
embeds it in PAML lower-triangle form in ``model/modelprotein.cpp`` (the
``model LG=`` block). The table must be identical for the model to be LG, so
this script reads that block from an IQ-TREE 2 source tree and writes a plain
whitespace file: 190 lower-triangle exchangeabilities (rows 1..19, columns
0..i-1, amino-acid order ARNDCQEGHILKMFPSTWYV) followed by 20 frequencies.

Usage: python make_lg.py <iqtree2-source-root>
"""
import os
import re
import sys


def extract(src_root):
    path = os.path.join(src_root, "model", "modelprotein.cpp")
    text = open(path).read()
    start = text.index("model LG=")
    body = text[start + len("model LG="):]
    body = body[: body.index(";")]
    nums = [float(t) for t in re.findall(r"[-+0-9.eE]+", body)]
    if len(nums) != 190 + 20:
        raise ValueError(f"expected 210 numbers in the LG block, found {len(nums)}")
    return nums


def main():
    if len(sys.argv) != 2:
        raise SystemExit("usage: python make_lg.py <iqtree2 source tree>")
    root = sys.argv[1]
    nums = extract(root)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lg.dat")
    with open(out, "w") as f:
        f.write("# LG exchangeabilities (PAML lower triangle, 190 values) then 20 frequencies\n")
        k = 0
        for i in range(1, 20):
            f.write(" ".join(repr(v) for v in nums[k:k + i]) + "\n")
            k += i
        f.write(" ".join(repr(v) for v in nums[190:]) + "\n")
    print("wrote", out)


if __name__ == "__main__":
    main()
