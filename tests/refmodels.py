"""Import the reference spatialpy package where it is present: the checkout
named by $SPATIALPY_REFERENCE, else its pip install in baseline/_ref.
Tests that need it skip without it."""
import os
import sys

import oracle

REF = oracle.reference_root()
STUBS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_stubs")


def spatialpy_or_skip():
    import pytest
    if REF is None:
        pytest.skip("reference package not present")
    sys.dont_write_bytecode = True
    for p in (STUBS, REF, os.path.join(REF, "test")):
        if p not in sys.path:
            sys.path.append(p)
    import spatialpy
    return spatialpy
