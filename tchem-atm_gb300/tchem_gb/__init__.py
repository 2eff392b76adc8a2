"""GB300 engine for TChem-atm's batched box-model TR-BDF2 time advance."""
