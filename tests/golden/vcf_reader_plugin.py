"""pytest plugin that runs TreeTime's own VCF reader tests (the reference's
test/test_vcf.py, reading tests only) against treetime_gb300.vcf.read_vcf:
after collection, each test module's ``read_vcf`` and ``TreeTimeError`` names
are pointed at this package's reader and exception class.  Used by
tests/test_vcf.py; needs the TreeTime sources (not shipped here)."""

import treetime_gb300.errors as _errors
import treetime_gb300.vcf as _vcf


def pytest_collection_modifyitems(session, config, items):
    for item in items:
        mod = getattr(item, "module", None)
        if mod is not None and hasattr(mod, "read_vcf"):
            mod.read_vcf = _vcf.read_vcf
            mod.TreeTimeError = _errors.TreeTimeError
