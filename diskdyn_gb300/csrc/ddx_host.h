// Host-side helpers shared by the readers of the reference's text files.
#pragma once

namespace ddx_host {

// The reference's tokeniser (tokenize_spaces with remove_quotes, src/read_in.cu:12-60):
// splits buf in place into at most `max` tokens at the separators '@', space, CR, LF and
// tab outside double quotes, then drops every double quote of each token.  Scanning stops
// once the max-th token has started, so that token runs to the end of the line.  tok needs
// room for max + 1 entries (the list ends with a null pointer).  Returns the token count.
int split(char* buf, char** tok, int max);

}  // namespace ddx_host
