"""Regenerate ``scattering_params.json`` from the reference's parameter modules.

The tables are published physical constants: the electron scattering
factor fits of Lobato & Van Dyck, Acta Cryst. A70 (2014) 636, the
five-Gaussian fits of International Tables for Crystallography Vol. C,
table 4.3.2.3, and the four-Gaussian Doyle & Turner, Acta Cryst. A24 (1968)
390 / Smith & Burge (1962) fits for Z = 1-98 (De Graef & McHenry, Structure of
Materials, table 12.1).  diffsims ships them as
``ATOMIC_SCATTERING_PARAMS_LOBATO`` (diffsims/utils/lobato_scattering_params.py:25),
``ATOMIC_SCATTERING_PARAMS`` (diffsims/utils/atomic_scattering_params.py:22),
element symbol -> five (a_i, b_i) pairs, and
``ATOMIC_SCATTERING_PARAMETERS_DOYLETURNER`` with the element symbols
``ELEMENTS`` (diffsims/structure_factor/atomic_scattering_parameters.py:24-60),
98 rows of a1-a4, b1-b4 in 1/Angstrom^2.  This script copies the numbers
verbatim into JSON so the library and the GPU host never need the reference.

Usage (needs a checkout of the reference; its path is the one argument)::

    python tests/golden/make_tables.py /path/to/diffsims-checkout

It writes ``diffsims_gb300/data/scattering_params.json``, the package's data
file (committed), and lives beside the test fixtures' generator because it is
a one-off build step, not part of the package.
"""
import importlib.util
import json
import pathlib
import sys


def _load_module(path, name):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def main(ref_root):
    ref = pathlib.Path(ref_root) / "diffsims" / "utils"
    lob = _load_module(ref / "lobato_scattering_params.py", "_lobato")
    xt = _load_module(ref / "atomic_scattering_params.py", "_xtables")
    dt = _load_module(pathlib.Path(ref_root) / "diffsims" / "structure_factor" / "atomic_scattering_parameters.py",
                      "_doyleturner")
    out = {
        "lobato": {k: [list(map(float, p)) for p in v]
                   for k, v in lob.ATOMIC_SCATTERING_PARAMS_LOBATO.items()},
        "xtables": {k: [list(map(float, p)) for p in v]
                    for k, v in xt.ATOMIC_SCATTERING_PARAMS.items()},
        "doyleturner": [list(map(float, row)) for row in dt.ATOMIC_SCATTERING_PARAMETERS_DOYLETURNER],
        "elements": list(dt.ELEMENTS),
    }
    dst = pathlib.Path(__file__).resolve().parents[2] / "diffsims_gb300" / "data" / "scattering_params.json"
    dst.write_text(json.dumps(out, sort_keys=True, separators=(",", ":")))
    print(f"wrote {dst} ({len(out['lobato'])} lobato, {len(out['xtables'])} xtables, "
          f"{len(out['doyleturner'])} doyle-turner)")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_tables.py /path/to/diffsims-checkout")
    main(sys.argv[1])
