"""torchtree CLI hooks of the GB300 plug-in."""
