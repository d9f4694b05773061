"""Collect the reference's own golden fixtures for the per-frequency path.

Run once in a checkout that has the HAMS-MREL reference next to it:

    python tests/golden/make_golden.py /path/to/HAMS-MREL

It copies, unchanged, the input decks and the expected HAMS/WAMIT-format
outputs (added mass and damping, excitation, and for the two examples the
motions and hydrostatics; for example5 a sample of the Hydrostar-format
files) of three reference cases into tests/golden/<case>/:

  config1   test/data/config1            3 bodies x 234 panels, h = 70 m,
                                         3 frequencies x 3 headings, IRSP = 0
                                         (the reference's integration test)
  example5  examples/example5_single_body  234 hull + 383 lid panels, h = 70 m,
                                         10 frequencies x 36 headings, IRSP = 1
  example3  examples/example3_multi_bodies_gen_mod
                                         2 bodies with lids and generalized
                                         modes, IRSP = 1

and the control file of the reference's GMRES integration test
(test/data/config1_gmres: config1's deck with Solver_type 2; its meshes are
config1's) into tests/golden/config1_gmres/.

The GPU machine has no copy of the reference, so the tests read only these
committed files.
"""
import os
import shutil
import sys

CASES = {
    "config1": ("test/data/config1/input", "test/data/config1/expected_output",
                ["OAMASS%d.txt", "ODAMPING%d.txt", "OEXFOR%d.txt"]),
    "example5": ("examples/example5_single_body/Input", "examples/example5_single_body/Output",
                 ["Hams_format/OAMASS%d.txt", "Hams_format/ODAMPING%d.txt", "Hams_format/OEXFOR%d.txt",
                  "Wamit_format/AmssDamp.1", "Wamit_format/ExcForce.3", "Wamit_format/Motion.4",
                  "Wamit_format/Hydrostat.hst"] +
                 ["Hydrostar_format/%s.rao" % f for f in (
                     "AddedMass_11", "AddedMass_15", "AddedMass_33", "WaveDamping_11", "WaveDamping_13",
                     "WaveDamping_33", "Excitation_1", "Excitation_3", "Excitation_5", "Motion_1", "Motion_3",
                     "Motion_5")]),
    "example3": ("examples/example3_multi_bodies_gen_mod/Input",
                 "examples/example3_multi_bodies_gen_mod/Output",
                 ["Hams_format/OAMASS%d.txt", "Hams_format/ODAMPING%d.txt", "Hams_format/OEXFOR%d.txt",
                  "Wamit_format/AmssDamp.1", "Wamit_format/ExcForce.3", "Wamit_format/Motion.4",
                  "Wamit_format/Hydrostat.hst"]),
}


def main(ref_root: str) -> None:
    here = os.path.dirname(os.path.abspath(__file__))
    for case, (inp, out, patterns) in CASES.items():
        dst_in = os.path.join(here, case, "input")
        dst_out = os.path.join(here, case, "expected")
        os.makedirs(dst_in, exist_ok=True)
        os.makedirs(dst_out, exist_ok=True)
        for name in sorted(os.listdir(os.path.join(ref_root, inp))):
            shutil.copy(os.path.join(ref_root, inp, name), os.path.join(dst_in, name))
        for pat in patterns:
            names = [pat % k for k in range(1, 7)] if "%d" in pat else [pat]
            for name in names:
                src = os.path.join(ref_root, out, name)
                if os.path.exists(src):
                    shutil.copy(src, os.path.join(dst_out, os.path.basename(name)))
    dst = os.path.join(here, "config1_gmres")
    os.makedirs(dst, exist_ok=True)
    shutil.copy(os.path.join(ref_root, "test/data/config1_gmres/input/ControlFile.in"),
                os.path.join(dst, "ControlFile.in"))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
