"""The command-line front end on the GPU: a NIfTI image through
`python -m decaes_gb300`-style arguments gives, in its .mat outputs, exactly
the arrays of the direct API call on the same image (and a B1 map file is
used as the flip angles)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_cli_matches_api(D, ctx, tmp_path):
    io = pytest.importorskip("scipy.io")
    from decaes_gb300 import cli, nifti
    X = (6, 5, 2)
    img = D.mock_image(D.MockImageOptions(MatrixSize=X, nTE=32, TE=10e-3, BackgroundFraction=0.3), seed=8)
    nifti.write(str(tmp_path / "mese.nii.gz"), img)
    args = [str(tmp_path / "mese.nii.gz"), "--T2map", "--T2part", "--TE", "10e-3", "--nT2", "40", "--T2Range", "10e-3",
            "2.0", "--SPWin", "10e-3", "25e-3", "--MPWin", "25e-3", "200e-3", "--Reg", "lcurve", "--nRefAngles", "16",
            "--Threshold", "200", "--SaveRegParam", "-o", str(tmp_path / "out"), "--quiet"]
    cli.run_main(args, ctx=ctx)
    mo = D.T2mapOptions(MatrixSize=X, nTE=32, TE=10e-3, nT2=40, T2Range=(10e-3, 2.0), Reg="lcurve", nRefAngles=16,
                        Threshold=200.0, SaveRegParam=True)
    po = D.T2partOptions.from_t2map(mo, SPWin=(10e-3, 25e-3), MPWin=(25e-3, 200e-3))
    maps, dist, parts = D.T2mapSEcorr_T2partSEcorr(np.asfortranarray(img, dtype=np.float64), mo, po, ctx=ctx)
    d = io.loadmat(str(tmp_path / "out" / "mese.t2dist.mat"))["dist"]
    np.testing.assert_array_equal(d, dist)
    m = io.loadmat(str(tmp_path / "out" / "mese.t2maps.mat"))
    for k in ("gdn", "ggm", "gva", "fnr", "snr", "alpha", "mu", "chi2factor"):
        np.testing.assert_array_equal(m[k], maps[k], err_msg=k)
    p = io.loadmat(str(tmp_path / "out" / "mese.t2parts.mat"))
    for k in ("sfr", "sgm", "mfr", "mgm"):
        np.testing.assert_array_equal(p[k], parts[k], err_msg=k)
    assert np.isfinite(d).any()


def test_cli_b1map(D, ctx, tmp_path):
    io = pytest.importorskip("scipy.io")
    from decaes_gb300 import cli, nifti
    X = (4, 4, 1)
    img = D.mock_image(D.MockImageOptions(MatrixSize=X, nTE=32, TE=10e-3), seed=9)
    b1 = np.random.default_rng(5).uniform(150, 180, size=X)
    nifti.write(str(tmp_path / "mese.nii"), img)
    nifti.write(str(tmp_path / "b1.nii"), b1)
    cli.run_main([str(tmp_path / "mese.nii"), "--T2map", "--TE", "10e-3", "--nT2", "40", "--T2Range", "10e-3", "2.0",
                  "--Reg", "none", "--B1map", str(tmp_path / "b1.nii"), "--quiet"], ctx=ctx)
    m = io.loadmat(str(tmp_path / "mese.t2maps.mat"))
    np.testing.assert_array_equal(m["alpha"], b1)


def test_daemon_on_gpu(D, ctx, tmp_path, monkeypatch):
    """The warm daemon serves two command lines with one context; results
    equal the direct API call's."""
    import socket
    import threading
    io = pytest.importorskip("scipy.io")
    from decaes_gb300 import daemon, nifti
    X = (5, 4, 2)
    img = D.mock_image(D.MockImageOptions(MatrixSize=X, nTE=32, TE=10e-3), seed=12)
    nifti.write(str(tmp_path / "a.nii"), img)
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    srv = daemon.make_server(port, ctx=ctx)
    th = threading.Thread(target=srv.serve_forever, daemon=True)
    th.start()
    try:
        monkeypatch.chdir(tmp_path)
        args = ["a.nii", "--T2map", "--TE", "10e-3", "--nT2", "40", "--T2Range", "10e-3", "2.0", "--Reg", "chi2",
                "--RegParams", "1.02", "--quiet"]
        assert daemon.run(args + ["-o", "r1"], port) == 0
        assert daemon.run(args + ["-o", "r2", "--precision", "mixed"], port) == 0
    finally:
        srv.shutdown()
        srv.server_close()
    mo = D.T2mapOptions(MatrixSize=X, nTE=32, TE=10e-3, nT2=40, T2Range=(10e-3, 2.0), Reg="chi2", Chi2Factor=1.02)
    maps, dist = D.T2mapSEcorr(np.asfortranarray(img, dtype=np.float64), mo, ctx=ctx)
    np.testing.assert_array_equal(io.loadmat(str(tmp_path / "r1" / "a.t2dist.mat"))["dist"], dist)
    assert (tmp_path / "r2" / "a.t2maps.mat").exists()


def test_daemon_clients_share_the_batching_server(D, ctx, tmp_path):
    """Four clients at once: their command lines run concurrently in the
    daemon and their T2map+T2part work goes to one continuous-batching server
    (decaes_server_*); every client's outputs equal the direct API call's."""
    import socket
    import threading
    io = pytest.importorskip("scipy.io")
    from decaes_gb300 import daemon, nifti
    X = (24, 20, 3)
    imgs = [D.mock_image(D.MockImageOptions(MatrixSize=X, nTE=32, TE=10e-3), seed=40 + i) for i in range(4)]
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    srv = daemon.make_server(port, ctx=ctx)
    th = threading.Thread(target=srv.serve_forever, daemon=True)
    th.start()
    args = ["img.nii", "--T2map", "--T2part", "--TE", "10e-3", "--nT2", "40", "--T2Range", "10e-3", "2.0", "--Reg",
            "chi2", "--RegParams", "1.02", "--SPWin", "10e-3", "25e-3", "--MPWin", "25e-3", "200e-3", "-o", "out",
            "--quiet"]
    status = {}

    def client(i):
        d = tmp_path / f"c{i}"
        d.mkdir()
        nifti.write(str(d / "img.nii"), imgs[i])
        status[i] = daemon.request({"cmd": "run", "cwd": str(d), "args": args}, port, timeout=300)

    try:
        ts = [threading.Thread(target=client, args=(i,)) for i in range(4)]
        for t in ts:
            t.start()
        for t in ts:
            t.join(timeout=300)
        sv = srv.solver().srv.stats()
    finally:
        srv.shutdown()
        srv.server_close()
    assert sv["completed"] == 4 and sv["failed"] == 0
    mo = D.T2mapOptions(MatrixSize=X, nTE=32, TE=10e-3, nT2=40, T2Range=(10e-3, 2.0), Reg="chi2", Chi2Factor=1.02)
    po = D.T2partOptions.from_t2map(mo, SPWin=(10e-3, 25e-3), MPWin=(25e-3, 200e-3))
    for i in range(4):
        assert status[i]["status"] == 0, status[i]["log"]
        maps, dist, parts = D.T2mapSEcorr_T2partSEcorr(np.asfortranarray(imgs[i], dtype=np.float64), mo, po, ctx=ctx)
        out = tmp_path / f"c{i}" / "out"
        np.testing.assert_array_equal(io.loadmat(str(out / "img.t2dist.mat"))["dist"], dist)
        np.testing.assert_array_equal(io.loadmat(str(out / "img.t2parts.mat"))["sfr"], parts["sfr"])
