"""Launchers (the counterparts of the reference's api/ scripts) on the CPU: the
shell launcher reaches the command line, and the warm daemon runs forwarded
command lines in the client's directory with one shared context, reports
failures by status, answers ping and stops on kill (GPU calls stubbed as in
test_cli.py)."""
import os
import socket
import subprocess
import threading

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_shell_launcher_help():
    sh = os.path.join(ROOT, "decaes.jl_gb300", "launchers", "decaes_gpu.sh")
    r = subprocess.run(["bash", sh, "--help"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "usage: decaes" in r.stdout


def test_daemon(D, tmp_path, monkeypatch, capsys):
    from decaes_gb300 import daemon
    from test_cli import BASE, _inputs, _Stubs
    st = _Stubs(monkeypatch)
    img, mask = _inputs(tmp_path)
    port = _free_port()
    srv = daemon.make_server(port, ctx=object(), batching=False)
    th = threading.Thread(target=srv.serve_forever, daemon=True)
    th.start()
    try:
        monkeypatch.chdir(tmp_path)  # relative paths are the client's
        rc = daemon.run(["img.nii.gz", "--mask", "mask.nii", "-o", "out", "--quiet"] + BASE, port)
        assert rc == 0
        assert (tmp_path / "out" / "img.t2maps.mat").exists() and (tmp_path / "out" / "img.t2dist.mat").exists()
        (kind, image, mo, b1), = st.calls
        np.testing.assert_array_equal(image, img * mask[..., None])
        rc = daemon.run(["img.nii.gz"], port)  # neither --T2map nor --T2part
        assert rc == 1 and "At least one of --T2map or --T2part" in capsys.readouterr().out
        assert daemon.main(["ping", "--port", str(port)]) == 0 and "2 runs served" in capsys.readouterr().out
        assert daemon.main(["kill", "--port", str(port)]) == 0
        th.join(timeout=10)
        assert not th.is_alive()
        assert daemon.main(["ping", "--port", str(port)]) == 3  # nothing listening any more
    finally:
        if th.is_alive():
            srv.shutdown()
        srv.server_close()


def test_daemon_runs_clients_concurrently(D, tmp_path, monkeypatch):
    """Two clients' command lines run at the same time in the daemon (a
    solver that lets neither finish until both have reached the GPU call),
    each in its own working directory and with its own log."""
    from decaes_gb300 import daemon
    from test_cli import BASE, _inputs, _Stubs
    meet = threading.Barrier(2, timeout=30)

    class MeetingSolver:
        def t2map(self, image, mo, b1):
            meet.wait()  # raises BrokenBarrierError after 30 s if the runs were serialized
            return _Stubs.maps(mo), _Stubs.dist(mo)

    port = _free_port()
    srv = daemon.make_server(port, ctx=object(), batching=False)
    monkeypatch.setattr(srv, "solver", lambda: MeetingSolver())
    th = threading.Thread(target=srv.serve_forever, daemon=True)
    th.start()
    dirs = [tmp_path / "a", tmp_path / "b"]
    results = {}

    def client(d):
        d.mkdir()
        _inputs(d)
        results[d.name] = daemon.request({"cmd": "run", "cwd": str(d),
                                          "args": ["img.nii.gz", "-o", "out"] + BASE}, port, timeout=60)

    try:
        ts = [threading.Thread(target=client, args=(d,)) for d in dirs]
        for t in ts:
            t.start()
        for t in ts:
            t.join(timeout=90)
        for d in dirs:
            r = results[d.name]
            assert r["status"] == 0, r["log"]
            assert (d / "out" / "img.t2maps.mat").exists()
            # each log names its own input file only
            assert str(d / "img.nii.gz") in r["log"]
            other = dirs[1 - dirs.index(d)]
            assert str(other / "img.nii.gz") not in r["log"]
    finally:
        srv.shutdown()
        srv.server_close()
