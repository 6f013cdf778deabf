"""Kernel interface mirroring tupan.lib (see extensions.py)."""
