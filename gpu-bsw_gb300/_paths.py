"""Locations of the package's sources and built libraries."""
import os

PKGDIR = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKGDIR, "csrc")
LIBDIR = os.path.join(PKGDIR, "_lib")
REPO = os.path.dirname(PKGDIR)
INCLUDE = os.path.join(REPO, "include")
GBSW_LIB = os.path.join(LIBDIR, "libgbsw.so")
