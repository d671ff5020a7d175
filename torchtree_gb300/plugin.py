"""torchtree plug-in entry (discovered through ``__plugin__``).

torchtree's ``PluginManager`` imports every top-level ``torchtree_*``
package and instantiates ``<package>.<__plugin__>``
(torchtree/cli/plugin_manager.py:10-23); the CLI then calls
``load_arguments`` on the sub-command parsers and
``process_tree_likelihood`` on each likelihood it writes
(torchtree/cli/plugin.py:4-16, torchtree/cli/evolution.py:697-698).
"""
from __future__ import annotations

from torchtree.cli.plugin import Plugin

from .cli.evolution import process_tree_likelihood as _retarget


class GB300(Plugin):
    def load_arguments(self, subparsers):
        for parser in subparsers.choices.values():
            parser.add_argument("--gb300", action="store_true",
                                help="evaluate tree likelihoods with the GB300 engine")
            parser.add_argument("--gb300-precision", dest="gb300_precision", choices=("f64", "f32"),
                                default="f64", help="partial precision of the GB300 engine")

    def process_tree_likelihood(self, arg, data):
        if getattr(arg, "gb300", False):
            _retarget(arg, data)
