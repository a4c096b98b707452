"""The autotuner's report format (include/hodlr3d.h, hodlr3d_autotune) as the
Python mirror reads it: engine timings, then the tensor-core launch shapes.
CPU only: the text is what product.cpp's autotune writes."""
from hodlr3d_gb300.hodlr3d import HODLR3D, parse_tune_report


def test_engine_rows_and_launch_shapes():
    text = ("transpose nrhs engine ms\n"
            "0 1 1 27.5\n0 1 2 7.4\n0 1 3 5.1\n1 32 3 46.2\n"
            "launch ta_split 1 2.9\nlaunch ta_split 4 2.4\nlaunch ta_split 32 2.6\n"
            "launch ta_split_chosen 4 2.4\n")
    rows, launch = parse_tune_report(text, HODLR3D.ENGINES)
    assert rows[0] == (False, 1, HODLR3D.ENGINES[1], 27.5)
    assert rows[-1] == (True, 32, HODLR3D.ENGINES[3], 46.2)
    assert len(rows) == 4
    assert launch == {"ta_split": {1: 2.9, 4: 2.4, 32: 2.6}, "ta_split_chosen": 4}


def test_empty_report_after_reps_zero():
    rows, launch = parse_tune_report("", HODLR3D.ENGINES)
    assert rows == [] and launch == {"ta_split": {}, "ta_split_chosen": None}
