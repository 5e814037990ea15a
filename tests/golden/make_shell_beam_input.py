"""Copies the reference's example model and design-variable inputs
(Working/shellBeamModelInput.yaml, Working/shellBeamDVarInput.yaml: its only input fixtures) next to
this script, unchanged, for the input-reader tests.

Usage: python make_shell_beam_input.py <path of the reference checkout>"""
import shutil
import sys
from pathlib import Path

if len(sys.argv) != 2:
    sys.exit(__doc__)
ref = Path(sys.argv[1]) / "Working"
here = Path(__file__).parent
shutil.copyfile(ref / "shellBeamModelInput.yaml", here / "shell_beam_model_input.yaml")
shutil.copyfile(ref / "shellBeamDVarInput.yaml", here / "shell_beam_dvar_input.yaml")
