"""python -m decaes_gb300 ...: the command-line front end (see cli.py)."""
from .cli import main

main()
