#!/usr/bin/env python
"""Command-line drop-in for the reference's reconstruct.py; see
mplicits_gb300/reconstruct.py."""

from mplicits_gb300.reconstruct import main

if __name__ == "__main__":
    main()
