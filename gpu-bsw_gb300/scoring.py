"""Scoring tables shared by the host API, the tests and the benchmark.

* ``AA_ORDER`` is the residue order of the reference's 24x24 protein matrix
  (``main.cpp:95`` of the reference; ``A R N D C Q E G H I L K M F P S T W Y V B Z X *``).
* ``encoding_table()`` builds the 91-entry ASCII -> matrix-index table that the
  reference's protein driver hard-codes (``driver.cpp:252-258``): each letter of
  ``AA_ORDER`` maps to its position, every other code below 91 (including the
  letters J, O and U) maps to 0, i.e. to ``A``.  Codes of 91 and above (``[``,
  lower-case letters, ...) are outside that table; the reference reads past it,
  this library rejects them.
* ``BLOSUM62`` is the standard published BLOSUM62 matrix (Henikoff & Henikoff,
  1992, half-bit units) in ``AA_ORDER``; the reference passes the same matrix
  from ``main.cpp:70-92``.
* ``DNA_SCORES_BENCH`` (+3/-3/-6/-1) is the scoring of the DNA benchmark
  workloads; ``DNA_SCORES_REFERENCE_CLI`` ({1,-3,-3,-1}) is what the reference's
  command line hard-codes (``main.cpp:210``).
"""

AA_ORDER = "ARNDCQEGHILKMFPSTWYVBZX*"

ENCODING_SIZE = 91
MATRIX_DIM = 24

DNA_SCORES_BENCH = (3, -3, -6, -1)
DNA_SCORES_REFERENCE_CLI = (1, -3, -3, -1)
AA_GAPS = (-6, -1)

_BLOSUM62_ROWS = """
 4 -1 -2 -2  0 -1 -1  0 -2 -1 -1 -1 -1 -2 -1  1  0 -3 -2  0 -2 -1  0 -4
-1  5  0 -2 -3  1  0 -2  0 -3 -2  2 -1 -3 -2 -1 -1 -3 -2 -3 -1  0 -1 -4
-2  0  6  1 -3  0  0  0  1 -3 -3  0 -2 -3 -2  1  0 -4 -2 -3  3  0 -1 -4
-2 -2  1  6 -3  0  2 -1 -1 -3 -4 -1 -3 -3 -1  0 -1 -4 -3 -3  4  1 -1 -4
 0 -3 -3 -3  9 -3 -4 -3 -3 -1 -1 -3 -1 -2 -3 -1 -1 -2 -2 -1 -3 -3 -2 -4
-1  1  0  0 -3  5  2 -2  0 -3 -2  1  0 -3 -1  0 -1 -2 -1 -2  0  3 -1 -4
-1  0  0  2 -4  2  5 -2  0 -3 -3  1 -2 -3 -1  0 -1 -3 -2 -2  1  4 -1 -4
 0 -2  0 -1 -3 -2 -2  6 -2 -4 -4 -2 -3 -3 -2  0 -2 -2 -3 -3 -1 -2 -1 -4
-2  0  1 -1 -3  0  0 -2  8 -3 -3 -1 -2 -1 -2 -1 -2 -2  2 -3  0  0 -1 -4
-1 -3 -3 -3 -1 -3 -3 -4 -3  4  2 -3  1  0 -3 -2 -1 -3 -1  3 -3 -3 -1 -4
-1 -2 -3 -4 -1 -2 -3 -4 -3  2  4 -2  2  0 -3 -2 -1 -2 -1  1 -4 -3 -1 -4
-1  2  0 -1 -3  1  1 -2 -1 -3 -2  5 -1 -3 -1  0 -1 -3 -2 -2  0  1 -1 -4
-1 -1 -2 -3 -1  0 -2 -3 -2  1  2 -1  5  0 -2 -1 -1 -1 -1  1 -3 -1 -1 -4
-2 -3 -3 -3 -2 -3 -3 -3 -1  0  0 -3  0  6 -4 -2 -2  1  3 -1 -3 -3 -1 -4
-1 -2 -2 -1 -3 -1 -1 -2 -2 -3 -3 -1 -2 -4  7 -1 -1 -4 -3 -2 -2 -1 -2 -4
 1 -1  1  0 -1  0  0  0 -1 -2 -2  0 -1 -2 -1  4  1 -3 -2 -2  0  0  0 -4
 0 -1  0 -1 -1 -1 -1 -2 -2 -1 -1 -1 -1 -2 -1  1  5 -2 -2  0 -1 -1  0 -4
-3 -3 -4 -4 -2 -2 -3 -2 -2 -3 -2 -3 -1  1 -4 -3 -2 11  2 -3 -4 -3 -2 -4
-2 -2 -2 -3 -2 -1 -2 -3  2 -1 -1 -2 -1  3 -3 -2 -2  2  7 -1 -3 -2 -1 -4
 0 -3 -3 -3 -1 -2 -2 -3 -3  3  1 -2  1 -1 -2 -2  0 -3 -1  4 -3 -2 -1 -4
-2 -1  3  4 -3  0  1 -1  0 -3 -4  0 -3 -3 -2  0 -1 -4 -3 -3  4  1 -1 -4
-1  0  0  1 -3  3  4 -2  0 -3 -3  1 -1 -3 -1  0 -1 -3 -2 -2  1  4 -1 -4
 0 -1 -1 -1 -2 -1 -1 -1 -1 -1 -1 -1 -1 -1 -2  0  0 -2 -1 -1 -1 -1 -1 -4
-4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4  1
"""

BLOSUM62 = tuple(int(x) for x in _BLOSUM62_ROWS.split())
assert len(BLOSUM62) == MATRIX_DIM * MATRIX_DIM


def encoding_table():
    """91-entry ASCII -> matrix index table (reference ``driver.cpp:252-258``)."""
    table = [0] * ENCODING_SIZE
    for idx, ch in enumerate(AA_ORDER):
        table[ord(ch)] = idx
    return tuple(table)


ENCODING = encoding_table()

# Amino-acid composition used to draw synthetic protein residues: the empirical
# frequencies of the 20 standard residues in the reference's protein test set
# (test-data/protein-query.fasta, 3,962,067 residues; the 534 'X' dropped and
# the rest renormalised), standing in for BLOSUM62 background frequencies.
AA_BACKGROUND = {
    "L": 0.08762, "A": 0.08183, "G": 0.07687, "V": 0.07519, "E": 0.06628,
    "S": 0.06455, "K": 0.06142, "T": 0.05983, "I": 0.05625, "D": 0.05579,
    "R": 0.04956, "P": 0.04299, "N": 0.04154, "F": 0.03846, "Q": 0.03818,
    "Y": 0.03518, "H": 0.02182, "M": 0.01955, "C": 0.01397, "W": 0.01299,
}
