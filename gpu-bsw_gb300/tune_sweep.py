"""Measures the built-in tuning table on the GPU: for each kind, length bin and
pair-count bucket, a synthetic batch of that many pairs of that bin is aligned
once per candidate kernel variant (gbsw_tune_device), and the bin's fastest
variant in each pass becomes its forward and its reverse entry.  Writes
``csrc/tuning_gb300.inc`` (the table every context starts with) and prints one
JSON line per entry.

    python -m gpu-bsw_gb300.tune_sweep            (from the repository root; needs a GPU)

The batches: DNA short bin -- references U[400,1024], queries U[150,300], 80%
mutated substrings (the DNA throughput shape); DNA long bin -- queries
U[1000,2048] against references U[1500,4096], all related (the long part of the
mixed batch); protein short bin -- lengths U[50,500]; protein long bin --
lengths U[512,1200]; 70% homologs.  Scoring +3/-3/-6/-1 and BLOSUM62 -6/-1.  The
open-ended last bucket is measured at 200,000 short pairs; for long pairs it
takes the choice of 60,000 (a larger long batch runs for seconds per candidate).
"""
import importlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "csrc", "tuning_gb300.inc")

# pairs per bucket: the bucket's upper edge, and a large batch for the last one
SHORT_COUNTS = (1000, 3000, 10000, 30000, 100000, 200000)
LONG_COUNTS = (1000, 3000, 10000, 30000, 60000)


def main():
    import torch
    gbsw = importlib.import_module("gpu-bsw_gb300")
    wl = importlib.import_module("gpu-bsw_gb300.workloads")
    importlib.import_module("gpu-bsw_gb300.build").build_all()
    dev = torch.device("cuda", 0)
    al = gbsw.Aligner(0)
    dna = gbsw.make_scoring(gbsw.DNA, scores=(3, -3, -6, -1))
    aa = gbsw.make_scoring(gbsw.PROTEIN, matrix=gbsw.scoring.BLOSUM62, gaps=(-6, -1))
    makers = {
        (0, 0): lambda n, s: wl.custom_dna(n, s, 400, 1024, 150, 300, related=0.8),
        (0, 1): lambda n, s: wl.custom_dna(n, s, 1500, 4096, 1000, 2048, related=1.0),
        (1, 0): lambda n, s: wl.custom_protein(n, s, 50, 500),
        (1, 1): lambda n, s: wl.custom_protein(n, s, 512, 1200),
    }
    table, rtable = {}, {}
    for (kind, b), make in makers.items():
        counts = LONG_COUNTS if b else SHORT_COUNTS
        for bucket, count in enumerate(counts):
            batch = make(count, 1000 + 10 * kind + b + 100 * bucket)
            d = [torch.from_numpy(x).to(dev) for x in (batch.ref, batch.ref_off, batch.query, batch.query_off)]
            ml = int(max(batch.ref_lengths().max(), batch.query_lengths().max()))
            rep = al.tune_device(dna if kind == 0 else aa, d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(),
                                 d[3].data_ptr(), batch.n, ml, reps=2)
            info = rep["bins"][b]
            names = [("dual%d" if c[0] else "int32_%d") % c[1] for c in rep["candidates"]]
            line = {"kind": "dna" if kind == 0 else "protein", "bin": b, "bucket": bucket, "pairs": info["pairs"],
                    "chosen": info["chosen"], "chosen_reverse": info["chosen_reverse"],
                    "ms_forward": dict(zip(names, [round(v, 3) for v in info["ms_forward"]])),
                    "ms_reverse": dict(zip(names, [round(v, 3) for v in info["ms_reverse"]]))}
            print(json.dumps(line), flush=True)
            if info["chosen"] and info["bucket"] == bucket:
                table[(kind, b, bucket)] = info["chosen"]
                rtable[(kind, b, bucket)] = info["chosen_reverse"]
            del d
            torch.cuda.empty_cache()
    al.close()
    for kind in (0, 1):
        for tab in (table, rtable):
            if (kind, 1, 4) in tab:
                tab[(kind, 1, 5)] = tab[(kind, 1, 4)]
    with open(OUT, "w") as f:
        f.write("// generated by gpu-bsw_gb300/tune_sweep.py on %s: t.variant (forward pass) and t.reverse\n"
                "// (reverse pass) [kind][bin][bucket] = {dual, lanes}\n" % torch.cuda.get_device_name(0))
        for name, tab in (("variant", table), ("reverse", rtable)):
            for (kind, b, bucket), (dual, lanes) in sorted(tab.items()):
                f.write("t.%s[%d][%d][%d] = gbsw_variant{%d, %d};\n" % (name, kind, b, bucket, dual, lanes))
    print(json.dumps({"written": OUT, "entries": len(table) + len(rtable)}))


if __name__ == "__main__":
    sys.exit(main())
