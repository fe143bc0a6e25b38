"""Writes tests/golden/real_image.npz from the reference's two real fixtures:
damascene/data/polynesia.ppm (321 x 481 RGB, the image Damascene's own
driver runs on) and labeledData/rio1_texton_codebook.yml (13 x 32 FP32, the
codebook src/SPFeatures.cpp:300-313 reads).

Stored: the image as H x W x 3 BGR uint8 (OpenCV's channel order, which
GlobalPbCuda packs), the codebook file's bytes as they are (so a test can
write it out and read it through gpb_load_codebook_yml) and the oracle's
texton labels of the image under that codebook.

Run in a tree where the reference is present:
    python tests/golden/make_golden_real.py [reference tree]
The reference tree defaults to $GPB_REFERENCE_TREE, else a "reference"
directory beside this repository.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def read_ppm(path):
    """Binary P6 with maxval 255 -> H x W x 3 RGB uint8."""
    with open(path, "rb") as f:
        data = f.read()
    fields, pos = [], 0
    while len(fields) < 4:
        while data[pos:pos + 1].isspace():
            pos += 1
        if data[pos:pos + 1] == b"#":
            pos = data.index(b"\n", pos) + 1
            continue
        end = pos
        while not data[end:end + 1].isspace():
            end += 1
        fields.append(data[pos:end])
        pos = end
    assert fields[0] == b"P6" and int(fields[3]) == 255, fields
    W, H = int(fields[1]), int(fields[2])
    pos += 1  # one whitespace byte after maxval
    return np.frombuffer(data[pos:pos + H * W * 3], np.uint8).reshape(H, W, 3)


def read_codebook_yml(text):
    """rows x cols FP32 matrix of an OpenCV FileStorage opencv-matrix."""
    head, body = text.split("data:", 1)
    rows = int(head.split("rows:")[1].split()[0])
    cols = int(head.split("cols:")[1].split()[0])
    vals = [float(v) for v in body.split("[", 1)[1].split("]", 1)[0].replace("\n", " ").split(",") if v.strip()]
    assert len(vals) == rows * cols
    return np.asarray(vals, np.float32).reshape(rows, cols)


def main():
    ref = (sys.argv[1] if len(sys.argv) > 1 else
           os.environ.get("GPB_REFERENCE_TREE") or os.path.join(os.path.dirname(ROOT), "reference"))
    import pyoracle as po
    rgb = read_ppm(os.path.join(ref, "damascene", "data", "polynesia.ppm"))
    bgr = np.ascontiguousarray(rgb[..., ::-1])
    with open(os.path.join(ref, "labeledData", "rio1_texton_codebook.yml"), "rb") as f:
        yml = f.read()
    cb = read_codebook_yml(yml.decode())
    tex = po.texton_map(po.grey_bgr(bgr), cb)
    np.savez_compressed(os.path.join(HERE, "real_image.npz"), bgr=bgr, codebook=cb,
                        codebook_yml=np.frombuffer(yml, np.uint8), texton=tex)
    print("real_image.npz: image %s, codebook %s, %d texton labels in use" %
          (bgr.shape, cb.shape, len(np.unique(tex))))


if __name__ == "__main__":
    main()
