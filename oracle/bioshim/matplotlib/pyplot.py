"""Empty matplotlib.pyplot stand-in (test-only)."""


def fill(*args, **kwargs):
    raise RuntimeError("plotting is not available in the test shim")
