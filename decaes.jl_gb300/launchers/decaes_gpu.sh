#!/usr/bin/env bash
# decaes_gpu.sh -- run the decaes command line on the GPU library (the
# counterpart of the reference's api/decaes.sh).  Arguments are those of the
# decaes CLI (see python -m decaes_gb300 --help), plus, first:
#   --python PATH   Python interpreter (default: python3)
#   --server        forward the command line to a running warm daemon
#                   (python -m decaes_gb300.daemon serve) instead of starting
#                   a new process; command lines forwarded at the same time
#                   run concurrently and share the daemon's batching server
#   --port P        the daemon's port (with --server)
set -e
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
pkg="$(dirname "$here")"   # the directory holding decaes_gb300/
py=python3
server=0
port=""
while [ $# -gt 0 ]; do
    case "$1" in
        --python) py="$2"; shift 2 ;;
        --server) server=1; shift ;;
        --port) port="--port $2"; shift 2 ;;
        *) break ;;
    esac
done
export PYTHONPATH="$pkg${PYTHONPATH:+:$PYTHONPATH}"
if [ "$server" = 1 ]; then
    exec "$py" -m decaes_gb300.daemon run $port -- "$@"
fi
exec "$py" -m decaes_gb300 "$@"
