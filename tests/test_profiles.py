"""The ncu and bench summaries under profiles/ are text, and every command
they quote runs files of this repository only (CPU only)."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PROFILES = os.path.join(ROOT, "profiles")


def test_profiles_are_short_text():
    names = sorted(os.listdir(PROFILES))
    assert names
    for n in names:
        assert n.endswith((".md", ".txt")), n
        assert os.path.getsize(os.path.join(PROFILES, n)) < 64 << 10, n


def test_profile_commands_name_files_of_the_repository():
    for n in sorted(os.listdir(PROFILES)):
        text = open(os.path.join(PROFILES, n)).read()
        for path in re.findall(r"[A-Za-z0-9_./-]+\.(?:py|sh|c|cu)\b", text):
            if path.startswith("gpurun_out/"):
                continue
            assert not path.startswith(("_work", "/")), (n, path)
            assert os.path.exists(os.path.join(ROOT, path)), (n, path)
