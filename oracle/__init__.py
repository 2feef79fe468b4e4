"""Test infrastructure: the CPU oracle and the recipes that build the reference's own code."""
import os
import re

_HERE = os.path.dirname(os.path.abspath(__file__))


def ref_include() -> str:
    """Where the reference's headers are: $QSF_REF_INCLUDE, else the default of the
    build recipe (REF_INCLUDE in oracle/Makefile, the one place that names it)."""
    env = os.environ.get("QSF_REF_INCLUDE")
    if env:
        return env
    try:
        with open(os.path.join(_HERE, "Makefile")) as f:
            m = re.search(r"^REF_INCLUDE\s*\?=\s*(\S+)", f.read(), re.M)
        return m.group(1) if m else ""
    except OSError:
        return ""
