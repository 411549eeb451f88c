"""The reference's bubble_2D test through the host driver on the GPU: main()
on the reference's deck and initial state writes test_solution/fi001.dat
after 100 steps, and in the exact form its payload is the reference golden's
bit for bit (SHA-256 of the big-endian values, as PETSc writes them).
"""
import json
import os

import pytest

import cases
import test_options
from golden.make_golden import digest
from taxila import options as O
from taxila import petsc_io
from taxila.lbm import main

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def test_reference_bubble_2d_deck_through_main(tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    p, run = O.params_from_options(O.parse_deck_text(test_options.DECK_2D))
    assert run.output_prefix == "test_solution/" and run.output_flow_fi
    main(test_options.DECK_2D, initialize_state=lambda p, run, w: cases.bubble_2d_reference_state(p),
         overrides={"exact": 1})
    assert os.path.exists(os.path.join("test_solution", "fi000.dat"))
    fi = petsc_io.read_vec(os.path.join("test_solution", "fi001.dat"))
    assert fi.size == p.nsites * p.ncomponents * p.Q
    with open(os.path.join(HERE, "golden", "bubble_2D_fi001.json")) as f:
        assert digest(fi) == json.load(f)["sha256_be"]
