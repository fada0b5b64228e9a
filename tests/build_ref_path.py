"""Import helper for tests that need the reference's sources (skips otherwise)."""
import os
import sys

import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import build_ref  # noqa: E402

if not build_ref.have_sources():
    pytest.skip("reference sources not available", allow_module_level=True)
