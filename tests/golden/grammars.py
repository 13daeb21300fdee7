"""Grammar texts shared by the fixture generator and the tests (plain data)."""

README_GRAMMAR = """E -> E + T [0.4]
E -> T [0.6]
T -> F * T [0.4]
T -> F [0.6]
F -> R ( V ) [0.3]
F -> V [0.7]
R -> sin [0.5]
R -> cos [0.5]
V -> X_0 [0.5]
V -> C [0.5]
"""

NOTATION_GRAMMAR = """E -> E + F [0.2]
E -> E - F [0.2]
E -> F [0.6]
F -> F * T [0.2]
F -> F / T [0.2]
F -> T [0.6]
T -> ( E ) P [0.1]
T -> R ( E ) [0.3]
T -> V [0.4]
T -> ( E ) [0.2]
V -> X_0 [0.2]
V -> X_1 [0.2]
V -> C [0.3]
V -> 5 [0.3]
R -> sin [0.2]
R -> cos [0.2]
R -> exp [0.2]
R -> sqrt [0.2]
R -> log [0.2]
P -> ^2 [0.25]
P -> ^3 [0.25]
P -> ^4 [0.25]
P -> ^5 [0.25]
"""

SAMPLING_GRAMMAR = """E -> E + F [0.2]
E -> E - F [0.2]
E -> F [0.6]
F -> F * T [0.2]
F -> F / T [0.2]
F -> T [0.6]
T -> ( E ) P [0.2]
T -> R ( E ) [0.2]
T -> V [0.4000000000000001]
T -> ( E ) [0.20000000000000004]
V -> X_0 [1.0]
R -> sin [0.2]
R -> cos [0.2]
R -> exp [0.2]
R -> sqrt [0.2]
R -> log [0.2]
P -> ^2 [1.0]
"""

BAD_GRAMMARS = {
    "no_arrow": "E X_0 [1.0]",
    "empty_lhs": "-> X_0 [1.0]",
    "two_arrows": "E -> X_0 -> 1 [1.0]",
    "no_prob": "E -> X_0",
    "no_close": "E -> X_0 [1.0",
    "two_close": "E -> X_0 [1.0]]",
    "two_lhs": "E F -> X_0 [1.0]",
    "bad_sum": "E -> X_0 [0.5]\nE -> 1 [0.4]",
    "undefined": "E -> A [1.0]",
    "empty": "",
}
