"""The ncu summaries under profiles/ name the command each was made with;
every such command runs committed files with options bench.py accepts
(host only: the options are checked against bench.py's parser)."""

import re
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def bench_options():
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--help"], capture_output=True, text=True,
                         timeout=120, check=True).stdout
    return set(re.findall(r"--[a-z0-9-]+", out))


def profile_commands():
    for path in sorted((ROOT / "profiles").glob("*.md")):
        text = path.read_text()
        # a command: "python bench.py ..." with its backslash continuations
        for match in re.finditer(r"python bench\.py((?:[^\n]*\\\n)*[^\n]*)", text):
            yield path.name, match.group(1)


def test_every_profile_names_its_command():
    for path in sorted((ROOT / "profiles").glob("*.md")):
        text = path.read_text()
        assert "Command" in text or "command" in text, path.name
        assert "ncu " in text or "rpg_smem_read_probe" in text or "bench.py" in text, path.name


def test_profile_commands_use_known_options():
    options = bench_options()
    commands = list(profile_commands())
    assert len(commands) >= 4
    for name, args in commands:
        used = set(re.findall(r"--[a-z0-9-]+", args))
        assert used <= options, (name, sorted(used - options))
