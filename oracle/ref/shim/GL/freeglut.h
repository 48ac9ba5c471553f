/* empty stand-in: the oracle uses no windowing */
#pragma once
