"""The profiling recipes committed under profiles/: every ncu command they
give leaves the GPU clocks alone (--clock-control none) and captures one
kernel (-k) with a few launches (-c), or only the one-pass launch list."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PROFILES = os.path.join(ROOT, "profiles")


def _commands():
    out = []
    for f in sorted(os.listdir(PROFILES)):
        if not f.endswith((".md", ".txt")):
            continue
        text = open(os.path.join(PROFILES, f)).read()
        # code blocks only, with continuation lines joined
        for block in re.findall(r"```(?:\w*)\n(.*?)```", text, re.S):
            joined = re.sub(r"\\\n\s*", " ", block)
            for line in joined.splitlines():
                if re.search(r"(^|[\s;&|])ncu\s", line):
                    out.append((f, line.strip()))
    return out


COMMANDS = _commands()


def test_profiles_hold_recipes():
    assert COMMANDS, "no ncu command found under profiles/"


@pytest.mark.parametrize("where,cmd", COMMANDS)
def test_ncu_commands_are_bounded_and_leave_clocks_alone(where, cmd):
    assert "--clock-control none" in cmd, where
    m = re.search(r"-c\s+(\d+)", cmd)
    launch_list = "--metrics gpu__time_duration.sum " in cmd + " "
    if "--set full" in cmd or "--section" in cmd or ("--metrics" in cmd and not launch_list):
        assert "-k " in cmd, f"{where}: a multi-pass capture names one kernel"
        assert m and int(m.group(1)) <= 5, f"{where}: a multi-pass capture takes a few launches"
    else:
        assert m, f"{where}: the launch list is bounded by -c"
