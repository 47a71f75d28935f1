"""Shared helpers of the test suite."""
import glob
import os

import numpy as np

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = sorted(glob.glob(os.path.join(HERE, "golden", "*.tsv.gz")))


def oracle_batch(batch, kind, scores=None, gaps=None):
    from importlib import import_module
    sc = import_module("gpu-bsw_gb300.scoring")
    if kind == 0:
        return oracle.align(oracle.DNA, batch.ref, batch.ref_off, batch.query, batch.query_off,
                            scores=scores)
    return oracle.align(oracle.AA, batch.ref, batch.ref_off, batch.query, batch.query_off,
                        matrix=sc.BLOSUM62, encoding=sc.ENCODING, gaps=gaps)


def first_mismatches(got, exp, limit=5):
    bad = np.nonzero(np.any(got != exp, axis=1))[0]
    return [(int(k), got[k].tolist(), exp[k].tolist()) for k in bad[:limit]], len(bad)
