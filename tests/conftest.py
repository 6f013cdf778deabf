"""Shared pytest configuration.

Markers:
  gpu  -- needs a CUDA device and the compiled library; run on the GPU machine
          with `python -m pytest tests -m gpu`.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: test needs a CUDA GPU (GB300)")
