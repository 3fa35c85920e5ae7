"""The documentation's pointers stay valid: every repository path quoted in the design doc,
INTEGRATION.md and README.md exists, and every profile summary names the command that made it."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DOCS = ["DESIGN.md", "INTEGRATION.md", "README.md"]
PREFIXES = ("sctl_gb300/", "tests/", "oracle/", "include/", "profiles/")


def test_quoted_paths_exist():
    missing = []
    for doc in DOCS:
        text = open(os.path.join(ROOT, doc)).read()
        for m in re.finditer(r"`([A-Za-z0-9_./-]+)`", text):
            p = m.group(1).rstrip(".")
            if p.startswith(PREFIXES) and not any(c in p for c in "*<>"):
                if not os.path.exists(os.path.join(ROOT, p)):
                    missing.append((doc, p))
    assert not missing, missing


def test_profile_summaries_name_their_command():
    for fn in os.listdir(os.path.join(ROOT, "profiles")):
        if fn.endswith(".md"):
            text = open(os.path.join(ROOT, "profiles", fn)).read()
            assert "Command" in text and "ncu" in text and "--clock-control none" in text, fn
