"""The five command lines: same argv and output lines as the reference's
toolkits (toolkits/*.cpp).  CPU: usage and exit code.  GPU: the first run's
output on the reference fixtures equals what the reference printed (the
exec_time line aside); CC/SSSP sparse-call counts are distinct vertices, so
only their dense-call counts and the summary are compared."""
import os
import re
import subprocess

import numpy as np
import pytest

import graphgen
from golden_util import Fixture, names

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(REPO, "geminigraph_gb300", "bin")

USAGE = {"bfs": "bfs [file] [vertices] [root]", "cc": "cc [file] [vertices]",
         "pagerank": "pagerank [file] [vertices] [iterations]", "sssp": "sssp [file] [vertices] [root]",
         "bc": "bc [file] [vertices] [root]"}


@pytest.mark.parametrize("app", sorted(USAGE))
def test_usage_line_and_exit_code(app):
    exe = os.path.join(BIN, app)
    if not os.path.exists(exe):
        pytest.skip("command lines not built")
    p = subprocess.run([exe], capture_output=True, text=True)
    assert p.stdout.strip() == USAGE[app]
    assert p.returncode == 255


def first_run(stdout):
    head, rest = stdout.split("exec_time=", 1)
    tail = rest.split("\n", 1)[1]
    nxt = re.split(r"active\(0\)|forward|delta\(0\)", tail)[0]
    return head, nxt


def write_files(tmp_path, fx):
    pu = tmp_path / (fx.name + ".bin")
    pw = tmp_path / (fx.name + ".wbin")
    pu.write_bytes(graphgen.to_records(fx.src, fx.dst))
    pw.write_bytes(graphgen.to_records(fx.src, fx.dst, fx.w))
    return str(pu), str(pw)


@pytest.mark.gpu
@pytest.mark.parametrize("name", names())
def test_cli_output_matches_reference(tmp_path, name):
    fx = Fixture(name)
    pu, pw = write_files(tmp_path, fx)
    V, root = str(fx.V), str(fx.root)

    def run(app, *args):
        p = subprocess.run([os.path.join(BIN, app)] + list(args), capture_output=True, text=True, timeout=300)
        assert p.returncode == 0, p.stderr
        assert p.stdout.count("exec_time=") == 6
        return first_run(p.stdout)

    head, summ = run("bfs", pu, V, root)
    assert head == fx.stdout("bfs") and summ == fx.summary("bfs")
    head, summ = run("pagerank", pu, V, "20")
    assert head == fx.stdout("pr") and summ == fx.summary("pr")
    head, summ = run("bc", pu, V, root)
    assert head == fx.stdout("bc") and summ == fx.summary("bc")
    head, summ = run("cc", pu, V)
    assert summ == fx.summary("cc")
    assert head.count("active(") == fx.stdout("cc").count("active(")
    head, summ = run("sssp", pw, V, root)
    assert summ == fx.summary("sssp")
    assert head.count("active(") == fx.stdout("sssp").count("active(")
