"""The Python example in README.md runs as written."""
import os
import re

import pytest

from conftest import REPO, gpu_available

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")]


def test_readme_python_example_runs(monkeypatch):
    text = open(os.path.join(REPO, "README.md")).read()
    blocks = re.findall(r"```python\n(.*?)```", text, re.S)
    assert blocks
    monkeypatch.chdir(REPO)
    ns = {}
    exec(compile(blocks[0], "README.md", "exec"), ns)
    assert ns["f"].result() == 95815104
    assert int(ns["b"].run()[-1]) > 0
