"""The EXR writer against the reference's own (write_openexr_image through
tinyexr): uncompressed files are byte-identical, including the HALF rounding
of exact ties (away from zero), subnormals, overflow and the YAR attributes;
ZIP files hold the same half values (the deflate stream itself may differ)."""
import os

import numpy as np

from conftest import golden
from yar_gb300 import exr

ATTRS = dict(spp=16, variance=0.25, input_file="cornell.pbrt", device="cpu")


def test_uncompressed_files_are_byte_identical(tmp_path):
    img = np.load(golden("cornell_c1_64.npz"))["image"]
    out = os.path.join(tmp_path, "a.exr")
    exr.write_exr(out, img, False, exr.yar_attributes(**ATTRS))
    assert open(out, "rb").read() == open(golden("exr_cornell_none.exr"), "rb").read()
    special = np.load(golden("exr_special_input.npy"))
    out = os.path.join(tmp_path, "s.exr")
    exr.write_exr(out, special, False, exr.yar_attributes(device="cpu"))
    assert open(out, "rb").read() == open(golden("exr_special_none.exr"), "rb").read()


def test_zip_files_hold_the_same_halves(tmp_path):
    img = np.load(golden("cornell_c1_64.npz"))["image"]
    ref_none, _ = exr.read_exr(golden("exr_cornell_none.exr"))
    ref_zip, attrs = exr.read_exr(golden("exr_cornell_zip.exr"))
    assert np.array_equal(ref_zip.view(np.uint32), ref_none.view(np.uint32))
    out = os.path.join(tmp_path, "z.exr")
    exr.write_exr(out, img, True, exr.yar_attributes(**ATTRS))
    mine, mattrs = exr.read_exr(out)
    assert np.array_equal(mine.view(np.uint32), ref_none.view(np.uint32))
    assert mattrs["compression"] == attrs["compression"]
    assert {k: v for k, v in mattrs.items()} == {k: v for k, v in attrs.items()}


def test_half_rounding():
    x = np.array([1.0, 65504.0, 65520.0, 1e-8, -0.0], np.float32)
    h = exr.to_half_bits(x)
    assert list(h) == [0x3C00, 0x7BFF, 0x7C00, 0x0000, 0x8000]
    # an exact tie rounds away from zero (0x3c8fd000 lies halfway between halves 0x247e and 0x247f)
    assert exr.to_half_bits(np.array([0x3C8FD000], np.uint32).view(np.float32))[0] == 0x247F


def test_cli_info(capsys):
    from yar_gb300.__main__ import main
    assert main(["info", golden("cornell_c1_64.yfs")]) == 0
    assert "triangles" in capsys.readouterr().out
