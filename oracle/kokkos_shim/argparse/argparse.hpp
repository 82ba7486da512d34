// argparse stand-in: the oracle driver does not parse command lines through the reference's Arguments.
#pragma once
