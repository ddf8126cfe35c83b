"""Write tests/golden/abi_layout_reference.json: the sizes, member offsets
and enumeration values that tests/c/abi_probe.c prints when compiled
against the reference's own headers (src/free_energy.h,
src/lb_data_options.h, src/field_options.h, src/hydro_options.h,
src/map.h, src/symmetric.h, src/blue_phase.h,
src/blue_phase_beris_edwards.h, src/phi_cahn_hilliard.h), so that the CPU
tests can check include/ludwig_gb.h against them where the reference is
absent.

    python tests/golden/make_abi_layout.py [/path/to/reference]
(default: $LUDWIG_REFERENCE_ROOT, else REF of oracle/ref.mk)
"""

import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402


def probe(include_args, defines=()):
    """Compile and run tests/c/abi_probe.c; return its JSON."""
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "probe")
        subprocess.run(["gcc", "-std=gnu11"] + list(defines) + include_args +
                       [os.path.join(ROOT, "tests", "c", "abi_probe.c"),
                        "-o", exe], check=True, capture_output=True)
        out = subprocess.run([exe], check=True, capture_output=True,
                             text=True).stdout
    return json.loads(out)


def reference_layout(ref_root):
    inc = ["-I" + os.path.join(ref_root, d) for d in ("src", "target",
                                                      "mpi_s")]
    return probe(inc, ("-DPROBE_REFERENCE", "-D_D3Q19_"))


def main(ref_root):
    layout = reference_layout(ref_root)
    with open(os.path.join(HERE, "abi_layout_reference.json"), "w") as fh:
        json.dump(layout, fh, indent=0, sort_keys=True)
    print("wrote abi_layout_reference.json:", len(layout), "entries")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else oracle.reference_root())
