"""Builds the oracle's C restatement (test infrastructure only)."""


def build() -> None:
    return None
