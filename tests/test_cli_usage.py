"""The command-line programs' argument handling (csrc/ug_cli.cpp), which runs before any
device work: usage on missing or unknown arguments, exit status 2, as the reference's
mains print their usage and stop."""
import subprocess

from unsupervised_growth_gb300 import build as B


def run(*args):
    B.build()
    return subprocess.run([B.CLI] + list(args), capture_output=True, text=True, timeout=60)


def test_usage():
    r = run()
    assert r.returncode == 2
    for prog in ("createNetworkForGrowth", "chainGrowth", "continueChainGrowth", "chainTest", "--track-inhibition"):
        assert prog in r.stderr


def test_bad_arguments():
    assert run("chainTest", "dir", "0", "4").returncode == 2                  # a positional argument missing
    assert run("chainGrowth", "a", "b", "c", "d", "--bogus", "1").returncode == 2
    r = run("createNetworkForGrowth", "cfg", "dir", "--n-ra")                  # an option without its value
    assert r.returncode == 2 and "needs a value" in r.stderr
    assert run("growSomething", "x").returncode == 2
    assert run("chainGrowth", "a", "b", "c", "d", "--save-long", "0").returncode == 2
