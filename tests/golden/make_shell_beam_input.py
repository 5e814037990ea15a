"""Copies the reference's example model input (Working/shellBeamModelInput.yaml, its only model
fixture) next to this script as shell_beam_model_input.yaml, unchanged, for the input-reader
tests.  Run in a checkout that has the reference tree at the given path."""
import shutil
import sys
from pathlib import Path

src = Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference") / "Working" / "shellBeamModelInput.yaml"
shutil.copyfile(src, Path(__file__).with_name("shell_beam_model_input.yaml"))
