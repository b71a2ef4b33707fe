"""Test fixtures: the reference's control files (decks/) and regression
checksums of the CPU restatement (oracle_runs.json)."""
import os

DECK_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "decks")


def deck_names():
    return sorted(n for n in os.listdir(DECK_DIR) if not n.startswith((".", "_")))


def deck_text(name):
    with open(os.path.join(DECK_DIR, name)) as f:
        return f.read()
