"""Copies the reference's example model and design-variable inputs
(Working/shellBeamModelInput.yaml, Working/shellBeamDVarInput.yaml: its only input fixtures) next to
this script, unchanged, for the input-reader tests.  Run in a checkout that has the reference
tree at the given path."""
import shutil
import sys
from pathlib import Path

ref = Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference") / "Working"
here = Path(__file__).parent
shutil.copyfile(ref / "shellBeamModelInput.yaml", here / "shell_beam_model_input.yaml")
shutil.copyfile(ref / "shellBeamDVarInput.yaml", here / "shell_beam_dvar_input.yaml")
