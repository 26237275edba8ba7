"""Warm-process front end: a local server that keeps one GPU context (its
stream, buffers and resident bases) across command-line runs, and the client
that forwards a command line to it.  The counterpart of the reference's
api/decaes_server.jl, which keeps a Julia process warm with DaemonMode so a
`decaes ...` call skips start-up and compilation; here a call skips Python and
CUDA start-up and reuses the bases already on the device.

    python -m decaes_gb300.daemon serve [--port P] [--device D] [--no-batching]
    python -m decaes_gb300.daemon run [--port P] -- <decaes arguments>
    python -m decaes_gb300.daemon ping | kill [--port P]

The server listens on 127.0.0.1 only.  Each client's command line runs in a
thread of its own, with relative paths taken from the client's working
directory and its log kept apart from the other runs'.  Their T2map (+
T2part) work goes to one continuous-batching server on the context
(decaes_server_*): command lines that arrive while others are on the GPU are
admitted and solved in the same ticks.  Runs with a B1 map and T2part-only
runs call the context directly (serialized with the ticks by the library).
With --no-batching every run calls the context directly.  The client prints
the run's log and exits with its status.  Protocol: one JSON line each way.
"""
from __future__ import annotations

import argparse
import io
import json
import logging
import os
import socket
import socketserver
import sys
import threading

DEFAULT_PORT = 45867


class BatchingSolver:
    """The GPU calls of the daemon's runs through one continuous-batching
    server on the shared context: a run submits its request and waits for
    it, and requests of concurrent runs share ticks."""

    def __init__(self, ctx):
        from . import cli
        from .server import Server
        self.ctx = ctx
        self.srv = Server(ctx)
        self.direct = cli.DirectSolver(ctx)

    def t2map_t2part(self, image, mo, po, b1):
        if b1 is not None:  # the server takes no B1 map
            return self.direct.t2map_t2part(image, mo, po, b1)
        return self.srv.result(self.srv.submit(image, mo, po))

    def t2map(self, image, mo, b1):
        if b1 is not None:
            return self.direct.t2map(image, mo, b1)
        return self.srv.result(self.srv.submit(image, mo, None))

    def t2part(self, dist, po):
        return self.direct.t2part(dist, po)

    def close(self):
        self.srv.close()


class _Server(socketserver.ThreadingMixIn, socketserver.TCPServer):
    allow_reuse_address = True
    daemon_threads = True

    def __init__(self, port: int, ctx, batching: bool = True):
        super().__init__(("127.0.0.1", port), _Handler)
        self.ctx = ctx
        self.runs = 0
        self.lock = threading.Lock()
        self.batching = batching
        self._solver = None

    def solver(self):
        from . import cli
        with self.lock:
            if self._solver is None:
                self._solver = BatchingSolver(self.ctx) if self.batching else cli.DirectSolver(self.ctx)
            return self._solver

    def server_close(self):
        super().server_close()
        if self._solver is not None and hasattr(self._solver, "close"):
            self._solver.close()
            self._solver = None


class _Handler(socketserver.StreamRequestHandler):
    def handle(self):
        from . import cli
        try:
            req = json.loads(self.rfile.readline().decode())
        except ValueError:
            return self._reply({"status": 2, "log": "bad request"})
        cmd = req.get("cmd", "run")
        if cmd == "ping":
            return self._reply({"status": 0, "log": f"decaes_gb300 daemon: {self.server.runs} runs served"})
        if cmd == "kill":
            self._reply({"status": 0, "log": "decaes_gb300 daemon stopped"})
            threading.Thread(target=self.server.shutdown, daemon=True).start()
            return None
        buf = io.StringIO()
        handler = logging.StreamHandler(buf)
        handler.setFormatter(logging.Formatter("[%(levelname)s] %(message)s"))
        handler.addFilter(cli.ThisThread())  # this run's records only
        status = 0
        cli.log.addHandler(handler)
        try:
            cli.run_main(list(req.get("args", [])), ctx=self.server.ctx, cwd=req.get("cwd") or os.getcwd(),
                         solver=self.server.solver())
        except SystemExit as e:  # argparse: --help, usage errors
            status = e.code if isinstance(e.code, int) else 1
        except Exception as e:
            buf.write(f"[ERROR] {type(e).__name__}: {e}\n")
            status = 1
        finally:
            cli.log.removeHandler(handler)
            with self.server.lock:
                self.server.runs += 1
        return self._reply({"status": status, "log": buf.getvalue()})

    def _reply(self, obj):
        self.wfile.write((json.dumps(obj) + "\n").encode())
        self.wfile.flush()


def make_server(port: int = DEFAULT_PORT, ctx=None, device: int = 0, batching: bool = True) -> _Server:
    """The server object (call serve_forever() on it); ctx defaults to a new
    context on `device`.  batching: the runs' GPU work goes through one
    continuous-batching server (else straight to the context)."""
    if ctx is None:
        from ._lib import Context
        ctx = Context(device)
    return _Server(port, ctx, batching)


def request(obj: dict, port: int = DEFAULT_PORT, timeout: float | None = None) -> dict:
    with socket.create_connection(("127.0.0.1", port), timeout=timeout) as s:
        s.sendall((json.dumps(obj) + "\n").encode())
        f = s.makefile("rb")
        line = f.readline()
    if not line:
        raise ConnectionError("no reply from the decaes_gb300 daemon")
    return json.loads(line.decode())


def run(args, port: int = DEFAULT_PORT) -> int:
    """Forward one decaes command line to the daemon; returns its status."""
    reply = request({"cmd": "run", "args": list(args), "cwd": os.getcwd()}, port)
    sys.stdout.write(reply.get("log", ""))
    return int(reply.get("status", 1))


def main(argv=None) -> int:
    argv = list(sys.argv[1:] if argv is None else argv)
    fwd = []
    if "--" in argv:
        i = argv.index("--")
        argv, fwd = argv[:i], argv[i + 1:]
    ap = argparse.ArgumentParser(prog="python -m decaes_gb300.daemon")
    ap.add_argument("command", choices=("serve", "run", "ping", "kill"))
    ap.add_argument("--port", type=int, default=DEFAULT_PORT)
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--no-batching", action="store_true", help="serve: run each command line straight on the context")
    a, rest = ap.parse_known_args(argv)
    if a.command == "serve":
        srv = make_server(a.port, device=a.device, batching=not a.no_batching)
        print(f"decaes_gb300 daemon on 127.0.0.1:{a.port} (GPU {a.device})", flush=True)
        try:
            srv.serve_forever()
        finally:
            srv.server_close()
        return 0
    try:
        if a.command == "run":
            return run(rest + fwd, a.port)
        reply = request({"cmd": a.command}, a.port, timeout=10)
        print(reply.get("log", ""))
        return int(reply.get("status", 1))
    except (ConnectionError, OSError) as e:
        print(f"decaes_gb300 daemon not reachable on port {a.port}: {e}", file=sys.stderr)
        return 3


if __name__ == "__main__":
    sys.exit(main())
