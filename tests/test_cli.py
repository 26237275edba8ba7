"""The command-line front end on the CPU (src/main.jl): argument handling,
file infos, the NIfTI / MAT / PAR-REC readers and writers, masks, BET, and the
processing flow with the GPU calls replaced by recording stubs (the GPU run of
the front end is in test_gpu_cli.py)."""
import os
import stat
import struct
import sys

import numpy as np
import pytest


@pytest.fixture
def cli(D):
    from decaes_gb300 import cli
    return cli


# ---- NIfTI ------------------------------------------------------------------
def test_nifti_roundtrip(D, tmp_path):
    from decaes_gb300 import nifti
    a = np.asfortranarray(np.random.default_rng(0).normal(size=(4, 5, 3, 7)))
    for name in ("a.nii", "a.nii.gz"):
        f = str(tmp_path / name)
        nifti.write(f, a)
        im = nifti.read(f)
        np.testing.assert_array_equal(im.raw, a)
        np.testing.assert_array_equal(im.scaled(), a)  # slope 0: unscaled


def test_nifti_scaling_follows_julia_promotion(D, tmp_path):
    """int16 voxels with Float32 slope/intercept are scaled in Float32."""
    from decaes_gb300 import nifti
    raw = np.arange(-30, 30, dtype=np.int16).reshape((3, 4, 5), order="F")
    f = str(tmp_path / "s.nii")
    nifti.write(f, raw, scl_slope=0.1, scl_inter=-2.5)
    got = nifti.read(f).scaled()
    want = raw.astype(np.float32) * np.float32(0.1) + np.float32(-2.5)
    assert got.dtype == np.float32
    np.testing.assert_array_equal(got, want)


def test_nifti2_header(D, tmp_path):
    from decaes_gb300 import nifti
    a = np.asfortranarray(np.arange(24, dtype=np.float32).reshape((2, 3, 4), order="F"))
    hdr = bytearray(540)
    struct.pack_into("<i", hdr, 0, 540)
    hdr[4:12] = b"n+2\x00\r\n\x1a\n"
    struct.pack_into("<hh", hdr, 12, 16, 32)
    struct.pack_into("<8q", hdr, 16, 3, 2, 3, 4, 1, 1, 1, 1)
    struct.pack_into("<q", hdr, 168, 544)
    struct.pack_into("<dd", hdr, 176, 2.0, 1.0)
    f = tmp_path / "n2.nii"
    f.write_bytes(bytes(hdr) + b"\x00" * 4 + a.tobytes(order="F"))
    im = nifti.read(str(f))
    np.testing.assert_array_equal(im.raw, a)
    got = im.scaled()
    assert got.dtype == np.float64  # NIfTI-2 scaling is Float64
    np.testing.assert_array_equal(got, a.astype(np.float64) * 2.0 + 1.0)


# ---- MAT --------------------------------------------------------------------
def test_mat_first_array_in_sorted_order(D, tmp_path, cli, caplog):
    pytest.importorskip("scipy.io")
    from decaes_gb300 import matfile
    rng = np.random.default_rng(1)
    b, a, m3 = rng.normal(size=(3, 3, 2, 5)), rng.normal(size=(3, 3, 2, 5)), rng.normal(size=(3, 3, 2))
    f = str(tmp_path / "img.mat")
    matfile.write(f, {"b": b, "a": a, "mask": m3})
    img = cli.load_image(f)
    np.testing.assert_array_equal(img, a)
    assert any("Choosing variable 'a'" in r.message for r in caplog.records)
    np.testing.assert_array_equal(cli.load_image(f, 3), m3)
    with pytest.raises(ValueError, match="No 2-D array"):
        matfile.read_array(f, 2)


# ---- PAR/REC ----------------------------------------------------------------
_PAR_COLUMNS = [
    ("slice number", "integer"), ("echo number", "integer"), ("dynamic scan number", "integer"),
    ("cardiac phase number", "integer"), ("image_type_mr", "integer"), ("scanning sequence", "integer"),
    ("index in REC file (in images)", "integer"), ("image pixel size (in bits)", "integer"),
    ("scan percentage", "integer"), ("recon resolution (x y)", "2*integer"), ("rescale intercept", "float"),
    ("rescale slope", "float"), ("scale slope", "float"), ("window center", "integer"), ("window width", "integer"),
    ("echo_time", "float"),
]


def _write_parrec(base, images, nx, ny, ri, rs, ss):
    """images: list of (slice, echo, pixel array (nx, ny) of ints); stored in reverse order."""
    lines = ["# === DATA DESCRIPTION FILE ===", "# === GENERAL INFORMATION ===",
             f".    Max. number of slices/locations    :   {max(s for s, _, _ in images)}",
             "# === IMAGE INFORMATION DEFINITION ===",
             "#  The rest of this file contains ONE line per image, this line contains the following information:", "#"]
    lines += [f"#  {n:<40} ({t})" for n, t in _PAR_COLUMNS]
    lines += ["#", "# === IMAGE INFORMATION ===", "#  sl ec ..."]
    order = list(range(len(images)))[::-1]
    rec = bytearray()
    for k, i in enumerate(order):
        rec += np.asarray(images[i][2], dtype="<i2").tobytes(order="F")
    for i, (sl, ec, _) in enumerate(images):
        idx = order.index(i)
        lines.append(f" {sl} {ec} 1 1 0 2 {idx} 16 100 {nx} {ny} {ri} {rs} {ss} 100 200 {10.0 * ec}")
    lines.append("# === END OF DATA DESCRIPTION FILE ===")
    (base.parent / (base.name + ".PAR")).write_text("\n".join(lines) + "\n")
    (base.parent / (base.name + ".REC")).write_bytes(bytes(rec))


def test_parrec(D, tmp_path, cli):
    nx, ny, ri, rs, ss = 4, 5, -3.0, 2.5, 0.125
    rng = np.random.default_rng(2)
    images = [(sl, ec, rng.integers(0, 4000, size=(nx, ny))) for sl in (1, 2) for ec in (1, 2, 3)]
    _write_parrec(tmp_path / "scan", images, nx, ny, ri, rs, ss)
    for name in ("scan.PAR", "scan.REC"):
        img = cli.load_image(str(tmp_path / name))
        assert img.shape == (nx, ny, 2, 3)
        for sl, ec, pv in images:
            np.testing.assert_allclose(img[:, :, sl - 1, ec - 1], (pv * rs + ri) / (rs * ss), rtol=1e-15)


def _write_xmlrec(base, images, nx, ny, ri, rs, ss):
    """The same images with a Philips XML header (one <Image_Info> per stored
    image: a <Key> with Slice/Echo/Dynamic/Phase/BValue/Grad Orient/Label
    Type/Type/Sequence/Index, then the image's attributes)."""
    def attr(name, typ, val):
        return f'<Attribute Name="{name}" Type="{typ}">{val}</Attribute>'
    order = list(range(len(images)))[::-1]
    rec = bytearray()
    for i in order:
        rec += np.asarray(images[i][2], dtype="<i2").tobytes(order="F")
    infos = []
    for i, (sl, ec, _) in enumerate(images):
        key = "".join([attr("Slice", "Int32", sl), attr("Echo", "Int32", ec), attr("Dynamic", "Int32", 1),
                       attr("Phase", "Int32", 1), attr("BValue", "Int32", 1), attr("Grad Orient", "Int32", 1),
                       attr("Label Type", "Enumeration", "-"), attr("Type", "Enumeration", "M"),
                       attr("Sequence", "Enumeration", "SE"), attr("Index", "Int32", order.index(i))])
        rest = "".join([attr("Pixel Size", "UInt16", 16), attr("Resolution X", "UInt16", nx),
                        attr("Resolution Y", "UInt16", ny), attr("Rescale Intercept", "Double", ri),
                        attr("Rescale Slope", "Double", rs), attr("Scale Slope", "Float", ss),
                        attr("Echo Time", "Float", 10.0 * ec)])
        infos.append(f"<Image_Info><Key>{key}</Key>{rest}</Image_Info>")
    xml = ('<?xml version="1.0" encoding="UTF-8"?><PRIDE_V5><Series_Info>' + attr("Max No Slices", "UInt16", 2) +
           "</Series_Info><Image_Array>" + "".join(infos) + "</Image_Array></PRIDE_V5>")
    (base.parent / (base.name + ".XML")).write_text(xml)
    (base.parent / (base.name + ".REC")).write_bytes(bytes(rec))


def test_xmlrec(D, tmp_path, cli):
    """An XML/REC pair reads as the same image as the PAR/REC pair of the same
    data (ParXRec.jl's XML form; no scanner file is available here, so the
    header follows the published layout written by _write_xmlrec)."""
    nx, ny, ri, rs, ss = 4, 5, -3.0, 2.5, 0.125
    rng = np.random.default_rng(5)
    images = [(sl, ec, rng.integers(0, 4000, size=(nx, ny))) for sl in (1, 2) for ec in (1, 2, 3)]
    (tmp_path / "p").mkdir()
    (tmp_path / "x").mkdir()
    _write_parrec(tmp_path / "p" / "scan", images, nx, ny, ri, rs, ss)
    _write_xmlrec(tmp_path / "x" / "scan", images, nx, ny, ri, rs, ss)
    want = cli.load_image(str(tmp_path / "p" / "scan.PAR"))
    for name in ("scan.XML", "scan.REC"):
        np.testing.assert_array_equal(cli.load_image(str(tmp_path / "x" / name)), want)


def test_ensure_ndims(D, cli, caplog):
    a = np.zeros((2, 2, 2, 3, 2))
    a[..., 0] = 1
    b = cli.ensure_ndims("x.nii", a, 4)
    assert b.shape == (2, 2, 2, 3) and (b == 1).all()
    assert any("selecting the first 4-D volume along dimension 5" in r.message for r in caplog.records)
    assert cli.ensure_ndims("x.nii", np.zeros((2, 3)), 4).shape == (2, 3, 1, 1)


# ---- arguments --------------------------------------------------------------
BASE = ["--T2map", "--TE", "10e-3", "--nT2", "40", "--T2Range", "10e-3", "2.0", "--Reg", "chi2", "--RegParams", "1.02"]


def test_parse_cli(D, cli, tmp_path):
    o = cli.parse_cli(["img.nii"] + BASE)
    assert o["Chi2Factor"] == 1.02 and o["T2map"] and not o["T2part"] and o["betargs"][0] == "-m"
    o = cli.parse_cli(["img.nii", "--T2map", "--Reg", "mdp", "--RegParams", "2.5", "--TE", "0.01"])
    assert o["NoiseLevel"] == 2.5
    o = cli.parse_cli(["img.nii", "--T2map", "--Reg", "chi2", "--Chi2Factor", "1.05"])  # deprecated spelling
    assert o["Chi2Factor"] == 1.05
    with pytest.raises(ValueError, match="both passed"):
        cli.parse_cli(["img.nii", "--T2map", "--Reg", "chi2", "--Chi2Factor", "1.05", "--RegParams", "1.02"])
    with pytest.raises(ValueError, match="At least one of --T2map or --T2part"):
        cli.parse_cli(["img.nii"])
    with pytest.raises(AssertionError, match="chi2 factor"):
        cli.parse_cli(["img.nii", "--T2map", "--Reg", "chi2"])
    settings = tmp_path / "settings.txt"
    settings.write_text("\n".join(["img.nii"] + BASE) + "\n")
    o = cli.parse_cli([f"@{settings}"])
    assert o["input"] == ["img.nii"] and o["nT2"] == 40 and o["T2Range"] == [0.01, 2.0]
    assert cli.clean_bet_args("-n,-f 0.25") == ["-m", "-n", "-f", "0.25"]


def test_file_infos(D, cli, tmp_path):
    o = cli.parse_cli(["d/a.nii", "e/b.nii.gz", "c.txt"] + BASE)
    fi = cli.get_file_infos(o)
    assert [f["outputfolder"] for f in fi] == ["d", "e"] and [f["choppedinputfile"] for f in fi] == ["a", "b"]
    fi = cli.get_file_infos(cli.parse_cli(["a.nii", "b.mat", "-o", "out"] + BASE))
    assert [f["outputfolder"] for f in fi] == ["out", "out"]
    with pytest.raises(ValueError, match="Incorrect number of output"):
        cli.get_file_infos(cli.parse_cli(["a.nii", "b.mat", "c.nii", "-o", "o1", "o2"] + BASE))
    with pytest.raises(ValueError, match="Number of mask files"):
        cli.get_file_infos(cli.parse_cli(["a.nii", "b.mat", "--mask", "m.nii"] + BASE))
    with pytest.raises(AssertionError, match="SetFlipAngle"):
        cli.get_file_infos(cli.parse_cli(["a.nii", "--B1map", "b1.nii", "--SetFlipAngle", "170"] + BASE))
    f = tmp_path / "settings.txt"
    f.write_text("x")
    with pytest.raises(ValueError, match="prepend an '@'"):
        cli.get_file_infos(cli.parse_cli([str(f)] + BASE))


# ---- processing flow with recording stubs -----------------------------------
class _Stubs:
    def __init__(self, monkeypatch):
        from decaes_gb300 import api
        self.calls = []

        def t2map(image, o, b1map=None, ctx=None):
            self.calls.append(("t2map", image.copy(), o, b1map))
            return self.maps(o), self.dist(o)

        def fused(image, mo, po, b1map=None, ctx=None):
            self.calls.append(("fused", image.copy(), mo, po, b1map))
            return self.maps(mo), self.dist(mo), self.parts(po)

        def t2part(dist, po, ctx=None):
            self.calls.append(("t2part", dist.copy(), po))
            return self.parts(po)

        monkeypatch.setattr(api, "T2mapSEcorr", t2map)
        monkeypatch.setattr(api, "T2mapSEcorr_T2partSEcorr", fused)
        monkeypatch.setattr(api, "T2partSEcorr", t2part)

    @staticmethod
    def maps(o):
        return {"t2times": np.geomspace(*o.T2Range, o.nT2), "gdn": np.full(o.MatrixSize, 2.0),
                "alpha": np.full(o.MatrixSize, 170.0)}

    @staticmethod
    def dist(o):
        return np.full(tuple(o.MatrixSize) + (o.nT2,), 0.5)

    @staticmethod
    def parts(po):
        return {k: np.full(po.MatrixSize, v) for k, v in (("sfr", 0.1), ("sgm", 0.02), ("mfr", 0.9), ("mgm", 0.08))}


def _inputs(tmp_path):
    from decaes_gb300 import nifti
    rng = np.random.default_rng(3)
    img = np.asfortranarray(rng.uniform(100, 1000, size=(4, 3, 2, 32)))
    mask = np.zeros((4, 3, 2))
    mask[1:3, :, :] = 1
    nifti.write(str(tmp_path / "img.nii.gz"), img)
    nifti.write(str(tmp_path / "mask.nii"), mask)
    return img, mask


def test_run_main_t2map_t2part(D, cli, tmp_path, monkeypatch):
    from decaes_gb300 import matfile
    st = _Stubs(monkeypatch)
    img, mask = _inputs(tmp_path)
    out = tmp_path / "out"
    settings = tmp_path / "opts.txt"
    settings.write_text("\n".join(["--SPWin", "10e-3", "25e-3", "--MPWin", "25e-3", "200e-3"]) + "\n")
    cli.run_main([str(tmp_path / "img.nii.gz"), "--mask", str(tmp_path / "mask.nii"), "-o", str(out), "--T2part",
                  "--quiet", f"@{settings}"] + BASE, ctx=object())
    (kind, image, mo, po, b1), = st.calls
    assert kind == "fused" and b1 is None
    np.testing.assert_array_equal(image, img * mask[..., None])
    assert mo.MatrixSize == (4, 3, 2) and mo.nTE == 32 and mo.nT2 == 40 and mo.Chi2Factor == 1.02
    assert po.SPWin == (10e-3, 25e-3) and po.nT2 == 40
    io = pytest.importorskip("scipy.io")
    d = io.loadmat(str(out / "img.t2dist.mat"))
    np.testing.assert_array_equal(d["dist"], st.dist(mo))
    m = io.loadmat(str(out / "img.t2maps.mat"))
    np.testing.assert_array_equal(m["gdn"], st.maps(mo)["gdn"])
    p = io.loadmat(str(out / "img.t2parts.mat"))
    np.testing.assert_array_equal(p["sfr"], st.parts(po)["sfr"])
    assert (out / "img.log").exists() and "Finished" in (out / "img.log").read_text()
    assert (out / "img.opts.txt").read_text() == settings.read_text()
    assert matfile is not None


def test_run_main_t2part_only_and_dry(D, cli, tmp_path, monkeypatch):
    from decaes_gb300 import nifti
    st = _Stubs(monkeypatch)
    dist = np.asfortranarray(np.random.default_rng(4).uniform(0, 1, size=(3, 3, 1, 40)))
    nifti.write(str(tmp_path / "dist.nii"), dist)
    cli.run_main([str(tmp_path / "dist.nii"), "--T2part", "--T2Range", "10e-3", "2.0", "--SPWin", "10e-3", "25e-3",
                  "--MPWin", "25e-3", "200e-3", "--dry", "--quiet"], ctx=object())
    (kind, d, po), = st.calls
    assert kind == "t2part" and po.nT2 == 40  # nT2 inferred from the distribution
    np.testing.assert_array_equal(d, dist)
    assert sorted(os.listdir(tmp_path)) == ["dist.nii"]  # a dry run writes nothing


def test_bad_file_does_not_stop_the_others(D, cli, tmp_path, monkeypatch):
    st = _Stubs(monkeypatch)
    _inputs(tmp_path)
    (tmp_path / "broken.nii").write_bytes(b"not a nifti file")
    cli.run_main([str(tmp_path / "broken.nii"), str(tmp_path / "img.nii.gz"), "-o", str(tmp_path / "o"), "--quiet"]
                 + BASE, ctx=object())
    assert len(st.calls) == 1
    assert "Error during processing of file" in (tmp_path / "o" / "broken.log").read_text()
    assert (tmp_path / "o" / "img.t2maps.mat").exists()


def test_bet_mask(D, cli, tmp_path, monkeypatch):
    """--bet runs the BET executable on the first echo and multiplies its mask in."""
    from decaes_gb300 import nifti
    st = _Stubs(monkeypatch)
    img, mask = _inputs(tmp_path)
    prepared = tmp_path / "prepared_mask.nii.gz"
    nifti.write(str(prepared), mask)
    bet = tmp_path / "fakebet"
    bet.write_text(f"#!{sys.executable}\nimport shutil, sys\n"
                   f"assert '-m' in sys.argv\nshutil.copyfile({str(prepared)!r}, sys.argv[2] + '_mask.nii.gz')\n")
    bet.chmod(bet.stat().st_mode | stat.S_IEXEC)
    cli.run_main([str(tmp_path / "img.nii.gz"), "--bet", "--betpath", str(bet), "--quiet", "--dry"] + BASE, ctx=object())
    (kind, image, mo, b1), = st.calls
    np.testing.assert_array_equal(image, img * mask[..., None])
