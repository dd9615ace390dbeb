"""The ncu summaries under profiles/: each states the command that made it,
every ncu command keeps the GPU clocks unlocked, and the commands run only
files of this repository's package and bench (no working files)."""
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _summaries():
    return sorted(glob.glob(os.path.join(ROOT, "profiles", "*.md")) + glob.glob(os.path.join(ROOT, "profiles", "*.txt")))


def test_profile_summaries_are_text_with_commands():
    files = _summaries()
    assert files
    for f in files:
        txt = open(f).read()
        assert len(txt) < 16384, f"{f}: a summary, not raw output"
        assert "ncu " in txt, f"{f}: no command"
        joined = re.sub(r"\\\n\s*", " ", txt)   # shell continuation lines
        for line in [ln for ln in joined.splitlines() if re.search(r"^\s*(\S+ )?ncu\b.*--", ln)]:
            assert "--clock-control none" in line, f"{f}: {line.strip()}"
        assert "_work/" not in txt, f"{f}: runs a working file"
        for script in re.findall(r"python (\S+\.py)", txt):
            assert os.path.exists(os.path.join(ROOT, script)), f"{f}: {script} is not in the repository"
    others = [p for p in glob.glob(os.path.join(ROOT, "profiles", "*")) if not p.endswith((".md", ".txt"))]
    assert not others, others
