"""The five workloads of this path as built models with pinned step counts.

``name`` selects the deck generator of exfem.decks; ``scale`` shrinks the
domain for oracle-sized cases.  io_interval is set exactly (the deck's save
interval only has to be no larger).
"""
from __future__ import annotations

from . import decks
from .model import Model

SPECS = {
    # name: (deck function, default steps, save every)
    "homogeneous_rectangle": (decks.homogeneous_rectangle, 4000, 1),
    "canyon": (decks.canyon, 8000, 4),
    "valley": (decks.valley, 20000, 10),
    "valley_batched": (decks.valley_batched, 20000, 10),
    "point_source": (decks.point_source, 4000, 4),
}


def build(name, scale=1.0, steps=None, save_every=None, **kw):
    fn, default_steps, default_save = SPECS[name]
    steps = default_steps if steps is None else int(steps)
    save_every = default_save if save_every is None else int(save_every)
    deck = fn(scale=scale, steps=steps, **kw)
    return Model(deck, nsteps=steps, io_interval=save_every)
