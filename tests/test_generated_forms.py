"""The generated 25-point bulk form is what its generator writes from the
in-tree distortion tables; the generator checks its shared-sum rewrite term
by term against the plain form before comparing."""
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_q25_header_up_to_date():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "oracle", "ref", "gen_q25_form.py"), "--check"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
