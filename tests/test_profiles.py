"""The profile summaries cite commands that still run: every
``python tests/kernel_cases.py <case>`` names a case the script
handles, every ``bench.py`` flag is one bench.py accepts, and every summary
gives its command (no GPU)."""

import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PROFILES = os.path.join(ROOT, "profiles")


def _summaries():
    return {f: open(os.path.join(PROFILES, f)).read() for f in sorted(os.listdir(PROFILES)) if f.endswith(".md")}


def test_every_summary_gives_a_command():
    for name, text in _summaries().items():
        assert "```" in text and ("ncu " in text or "bench.py" in text), name
        for line in text.splitlines():
            if line.startswith("ncu --"):
                assert "--clock-control none" in line, f"{name}: {line[:80]}"


def test_cited_kernel_cases_exist():
    src = open(os.path.join(ROOT, "tests", "kernel_cases.py")).read()
    known = set(re.findall(r'which == "([a-z0-9]+)"', src)) | set(re.findall(r'which in \(([^)]*)\)', src))
    known = {k.strip(' "') for item in known for k in item.split(",")}
    for name, text in _summaries().items():
        for case in re.findall(r"tests/kernel_cases\.py ([a-z0-9]+)", text):
            assert case in known, f"{name}: kernel case {case!r} is not in kernel_cases.py"


def test_cited_bench_flags_exist():
    src = open(os.path.join(ROOT, "bench.py")).read()
    flags = set(re.findall(r'add_argument\("(--[a-z0-9-]+)"', src))
    for name, text in _summaries().items():
        for cmd in re.findall(r"bench\.py((?: --[a-z0-9-]+(?: [a-z0-9.]+)?)+)", text):
            for flag in re.findall(r"--[a-z0-9-]+", cmd):
                assert flag in flags, f"{name}: bench.py has no {flag}"
