"""String labels with prime levels (host-only), restating tncontract/label.py.

A primed label remembers the label it was primed from (its parent), so that
priming is reversible: ``Label.__init__`` / ``parent`` / ``origin`` /
``parents`` follow ``label.py:17-61`` and the module functions
``label.py:64-92``.
"""
from __future__ import annotations

import uuid

__all__ = ['prime_label', 'unprime_label', 'noprime_label', 'prime_level',
           'unique_label']


class Label(str):
    """A ``str`` that carries the label it was primed from (``label.py:17``)."""

    def __new__(cls, value, **kwargs):
        return str.__new__(cls, value)

    def __init__(self, label, parent=None):
        self._parent = parent
        if isinstance(label, Label) and parent is None:
            self._parent = label._parent

    @property
    def parent(self):
        return self._parent

    @property
    def origin(self):
        node = self
        while hasattr(node, "parent"):
            node = node.parent
        return node

    @property
    def parents(self):
        level, node = 0, self
        while hasattr(node, "parent") and node.parent is not None:
            node = node.parent
            level += 1
        return level


def prime_label(label, prime="'"):
    """``label.py:64-66``"""
    return Label(str(label) + prime, parent=label)


def unprime_label(label, prime="'"):
    """``label.py:69-78``"""
    try:
        parent = label.parent
    except AttributeError:
        raise ValueError("label is not primed")
    if str(parent) + prime == label:
        return parent
    raise ValueError("label is not primed with \"" + prime + "\"")


def noprime_label(label):
    """``label.py:81-86``"""
    try:
        return label.origin
    except AttributeError:
        return label


def prime_level(label):
    """``label.py:84-88``"""
    try:
        return label.parents
    except AttributeError:
        return 0


def unique_label():
    """``label.py:90-92``: a random UUID string."""
    return str(uuid.uuid4())
