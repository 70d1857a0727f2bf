"""Locations of the in-tree native libraries."""
import os

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC_DIR = os.path.join(PKG_DIR, "csrc")
INCLUDE_DIR = os.path.join(REPO_DIR, "include")
GBSA_SO = os.path.join(PKG_DIR, "libgbsa.so")
SYNTH_SO = os.path.join(PKG_DIR, "libgbsa_synth.so")
ORACLE_DIR = os.path.join(REPO_DIR, "oracle")
ORACLE_SO = os.path.join(ORACLE_DIR, "liboracle.so")
