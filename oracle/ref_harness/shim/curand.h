/* host stand-in: only the type names used in declarations */
#pragma once
