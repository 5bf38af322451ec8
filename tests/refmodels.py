"""Import the reference spatialpy package where its sources are present
(CPU tests in the development container only; never on the GPU machine)."""
import os
import sys

REF = os.environ.get("SPATIALPY_REFERENCE", "/root/reference")
STUBS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_stubs")


def spatialpy_or_skip():
    import pytest
    if not os.path.isdir(os.path.join(REF, "spatialpy")):
        pytest.skip("reference sources not present")
    sys.dont_write_bytecode = True
    for p in (STUBS, REF, os.path.join(REF, "test")):
        if p not in sys.path:
            sys.path.append(p)
    import spatialpy
    return spatialpy
