"""Generate the golden fixtures in this folder from the reference checkout.

Run here (where the reference checkout and oracle/_ref exist):
    python tests/golden/make_golden.py /path/to/STAQ-DIC   (or STAQDIC_REFERENCE=...)

Writes
  circular_hole_pair.npz  the shipped 400x400 plate-with-hole pair (frames 000
      and 001 with their masks, decoded from the PackBits TIFFs) and, from
      ``results_Circular_hole 040_ws32_st16.mat``, the quadtree DICmesh (with
      the uniform grid x0, y0 it was refined from, elementMinSize and the
      hanging-node list irregular) and the reference's final U, F and
      ALSub1BadPtNum for that pair.
  ba_interp2_golden.npz   inputs and outputs of the reference's own
      ba_interp2.cpp (compiled unmodified in oracle/_ref) in double and single.
"""
import os
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def _packbits(data, nbytes):
    out = bytearray()
    i = 0
    while len(out) < nbytes and i < len(data):
        n = data[i]
        i += 1
        if n < 128:
            out += data[i:i + n + 1]
            i += n + 1
        elif n > 128:
            out += bytes([data[i]]) * (257 - n)
            i += 1
    return bytes(out[:nbytes])


def read_tiff_u8(path):
    """8-bit grayscale TIFF (uncompressed or PackBits) -> array [row, col]."""
    b = open(path, "rb").read()
    bo = "<" if b[:2] == b"II" else ">"
    off = struct.unpack(bo + "I", b[4:8])[0]
    n = struct.unpack(bo + "H", b[off:off + 2])[0]
    tags = {}
    for i in range(n):
        e = b[off + 2 + 12 * i: off + 14 + 12 * i]
        tag, typ, cnt = struct.unpack(bo + "HHI", e[:8])
        size = {1: 1, 3: 2, 4: 4}.get(typ, 4) * cnt
        raw = e[8:12] if size <= 4 else b[struct.unpack(bo + "I", e[8:12])[0]:][:size]
        fmt = {1: "B", 3: "H", 4: "I"}.get(typ, "I")
        tags[tag] = list(struct.unpack(bo + fmt * cnt, raw[:struct.calcsize(fmt) * cnt]))
    W, H = tags[256][0], tags[257][0]
    assert tags.get(258, [8])[0] == 8 and tags.get(277, [1])[0] == 1
    comp = tags.get(259, [1])[0]
    rps = tags.get(278, [H])[0]
    out = bytearray()
    for so, sc in zip(tags[273], tags[279]):
        rows = min(rps, H - len(out) // W)
        chunk = b[so:so + sc]
        out += _packbits(chunk, rows * W) if comp == 32773 else chunk[:rows * W]
    img = np.frombuffer(bytes(out), dtype=np.uint8).reshape(H, W)
    if tags.get(262, [1])[0] == 0:  # WhiteIsZero
        img = 255 - img
    return img


def main(ref):
    import scipy.io as sio
    imgdir = os.path.join(ref, "img_syn_circular_hole")
    mskdir = os.path.join(ref, "img_syn_circular_hole_maskfiles")
    raw_f = read_tiff_u8(os.path.join(imgdir, "Circular_hole 000.tif"))
    raw_g = read_tiff_u8(os.path.join(imgdir, "Circular_hole 001.tif"))
    mf = read_tiff_u8(os.path.join(mskdir, "img_syn_circular_hole_maskfiles0000.tif"))
    mg = read_tiff_u8(os.path.join(mskdir, "img_syn_circular_hole_maskfiles0001.tif"))
    m = sio.loadmat(os.path.join(ref, "results_Circular_hole 040_ws32_st16.mat"),
                    squeeze_me=True, struct_as_record=False)
    dm, dp = m["DICmesh"], m["DICpara"]
    # MATLAB stores Img = imread(...)' : Img(x, y) = raw[y, x]  -> arrays (W, H)
    np.savez_compressed(
        os.path.join(HERE, "circular_hole_pair.npz"),
        f=raw_f.T.copy(order="F"), g=raw_g.T.copy(order="F"),
        maskf=(mf.T != 0).astype(np.uint8), maskg=(mg.T != 0).astype(np.uint8),
        ImgRefMask=np.asarray(dp.ImgRefMask, dtype=np.uint8),
        coordinatesFEM=np.asarray(dm.coordinatesFEM, dtype=np.float64),
        elementsFEM=np.asarray(dm.elementsFEM, dtype=np.int32),
        dirichlet=np.asarray(dm.dirichlet, dtype=np.int32),
        markCoordHoleEdge=np.asarray(dm.markCoordHoleEdge, dtype=np.int32),
        U=np.asarray(m["ResultDisp"][0].U, dtype=np.float64),
        F=np.asarray(m["ResultDefGrad"][0].F, dtype=np.float64),
        ALSub1BadPtNum=np.asarray(m["ResultDisp"][0].ALSub1BadPtNum, dtype=np.int32),
        winsize=np.int32(dp.winsize), winstepsize=np.int32(dp.winstepsize),
        # GenerateQuadtreeMesh's input (the uniform MeshSetUp grid and
        # elementMinSize) and its hanging-node list
        x0=np.asarray(dm.x0, dtype=np.float64), y0=np.asarray(dm.y0, dtype=np.float64),
        elementMinSize=np.float64(dm.elementMinSize),
        irregular=np.asarray(dm.irregular, dtype=np.int32).reshape(-1, 3))

    from oracle import oracle as orc
    from oracle import build as ob
    ob.build_ref(force=True)
    rng = np.random.default_rng(20240601)
    M, N = 37, 29
    F64 = np.asfortranarray(rng.normal(size=(M, N)))
    # points inside, on integer nodes, near and beyond every border (clamping)
    X = np.concatenate([rng.uniform(-3, N + 4, 400), np.arange(1, N + 1, dtype=float),
                        rng.uniform(3, N - 3, 200)])
    Y = np.concatenate([rng.uniform(-3, M + 4, 400), rng.uniform(1, M, N),
                        rng.uniform(3, M - 3, 200)])
    Z64 = orc.ref_ba_interp2(F64, X, Y)
    F32 = F64.astype(np.float32)
    Z32 = orc.ref_ba_interp2(F32, X.astype(np.float32), Y.astype(np.float32))
    np.savez_compressed(os.path.join(HERE, "ba_interp2_golden.npz"), F=F64, X=X, Y=Y, Z64=Z64,
                        Z32=Z32)
    print("wrote fixtures")


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("STAQDIC_REFERENCE")
    if not ref or not os.path.isdir(ref):
        sys.exit("make_golden.py: give the STAQ-DIC checkout as the first argument or in "
                 "STAQDIC_REFERENCE (got %r)" % (ref,))
    main(ref)
